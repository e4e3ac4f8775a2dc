"""Helpers shared by the tests: golden fixtures and output canonicalisation."""
from __future__ import annotations

import hashlib
import json
from functools import lru_cache
from pathlib import Path

GOLDEN = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=1)
def golden() -> dict:
    return json.loads((GOLDEN / "cases.json").read_text())


def kat(name: str) -> dict:
    return next(c for c in golden()["kat"] if c["name"] == name)


def synth_case(name: str) -> dict:
    return next(c for c in golden()["synth"] if c["name"] == name)


def kat_text(name: str) -> bytes:
    return (GOLDEN / ("kat_%s.fa" % name)).read_bytes()


def synth_case_text(name: str) -> bytes:
    from cases import SYNTH_CASES, synth_text
    case = next(c for c in SYNTH_CASES if c["name"] == name)
    text = synth_text(case)
    want = synth_case(name)["fasta_sha256"]
    got = hashlib.sha256(text).hexdigest()
    assert got == want, "synthetic input %s differs from the fixture's (generator drift)" % name
    return text


def sorted_lines(path) -> list[str]:
    lines = Path(path).read_text().splitlines()
    return sorted(lines, key=lambda s: int(s.split()[0]))


def sha_lines(lines: list[str]) -> str:
    return hashlib.sha256(("\n".join(lines) + ("\n" if lines else "")).encode()).hexdigest()


def node_lines(keys, mult) -> list[str]:
    """graph.cpp:569 node lines from (key, 8 multiplicities) records."""
    acgt = "ACGT"
    out = []
    for key, m in zip(keys.tolist(), mult.tolist()):
        arcs = " ".join((acgt[s & 3] if m[s] else "") + "#" for s in range(8))
        out.append("%d %s %s" % (key, arcs, " ".join(str(v) for v in m)))
    return out
