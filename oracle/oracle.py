"""Python binding of the CPU restatement (liboracle.so) and runners for the
reference binaries built from the reference's own sources (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, always as the checker or the timed CPU
baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "build" / "liboracle.so"
ORACLE_BIN = HERE / "build" / "swap_oracle"
REF_SWAP = HERE / "_ref" / "swap"
REF_DUMP = HERE / "_ref" / "ref_dump"
REF_CONTIGS = HERE / "_ref" / "ref_contigs"

ERRORS = {0: "ok", -1: "no record start", -2: "unterminated record", -3: "NUL byte",
          -4: "bad k", -5: "out of memory"}


class OracleReads(C.Structure):
    _fields_ = [("codes", C.c_void_p), ("off", C.c_void_p), ("len", C.c_void_p),
                ("n_reads", C.c_uint64), ("n_bases", C.c_uint64), ("n_records", C.c_uint64)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            subprocess.run(["make", "-s", "-C", str(HERE), "restatement"], check=True)
        L = C.CDLL(str(LIB_PATH))
        P, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
        L.oracle_parse_fasta.argtypes = [C.c_char_p, u64, i32, C.POINTER(OracleReads)]
        L.oracle_parse_fasta.restype = i32
        L.oracle_reads_free.argtypes = [C.POINTER(OracleReads)]
        L.oracle_build.argtypes = [C.POINTER(OracleReads), i32, i32, i32, i32]
        L.oracle_build.restype = P
        L.oracle_graph_size.argtypes = [P]
        L.oracle_graph_size.restype = u64
        L.oracle_graph_get.argtypes = [P, P, P]
        L.oracle_graph_free.argtypes = [P]
        L.oracle_write_kmer_graph.argtypes = [P, i32, C.c_char_p]
        L.oracle_write_node_lines.argtypes = [P, C.c_char_p]
        L.oracle_graph_stats.argtypes = [P, i32, C.POINTER(C.c_int64)]
        L.oracle_kmer_graph_neighbour.argtypes = [u64, i32, i32]
        L.oracle_kmer_graph_neighbour.restype = u64
        L.oracle_revcomp.argtypes = [u64, i32]
        L.oracle_revcomp.restype = u64
        L.oracle_merge.argtypes = [i32, u64, P, P, P, i32, C.POINTER(C.c_void_p),
                                   C.POINTER(u64), C.POINTER(u64)]
        L.oracle_merge.restype = i32
        L.oracle_free_text.argtypes = [P]
        L.oracle_merge_tree_order.argtypes = [i32, u64, P, P, P]
        L.oracle_merge_tree_order.restype = i32
        L.oracle_prune.argtypes = [i32, C.c_char_p, u64, P, i32, C.POINTER(C.c_void_p), C.POINTER(u64),
                                   C.POINTER(u64)]
        L.oracle_prune.restype = i32
        L.oracle_simplify_lines.argtypes = [i32, C.c_char_p, u64, P, C.POINTER(C.c_void_p), C.POINTER(u64),
                                            C.POINTER(u64)]
        L.oracle_simplify_lines.restype = i32
        L.oracle_lines_tree_order.argtypes = [i32, C.c_char_p, u64, P, u64, C.POINTER(u64)]
        L.oracle_lines_tree_order.restype = i32
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code: int):
        super().__init__("oracle: %s" % ERRORS.get(code, code))
        self.code = code


def parse(text: bytes, k: int) -> dict:
    """Framing + normalisation; returns codes/off/len numpy copies."""
    r = OracleReads()
    e = lib().oracle_parse_fasta(text, len(text), k, C.byref(r))
    if e:
        raise OracleError(e)
    try:
        out = {
            "n_reads": r.n_reads, "n_bases": r.n_bases, "n_records": r.n_records,
            "codes": np.ctypeslib.as_array((C.c_uint8 * max(r.n_bases, 1)).from_address(r.codes))[: r.n_bases].copy(),
            "off": np.ctypeslib.as_array((C.c_uint64 * max(r.n_reads, 1)).from_address(r.off))[: r.n_reads].copy(),
            "len": np.ctypeslib.as_array((C.c_uint32 * max(r.n_reads, 1)).from_address(r.len))[: r.n_reads].copy(),
        }
    finally:
        lib().oracle_reads_free(C.byref(r))
    return out


class OracleGraph:
    def __init__(self, handle: int, k: int):
        self._h = C.c_void_p(handle)
        self.k = k

    def __del__(self):
        if self._h:
            lib().oracle_graph_free(self._h)
            self._h = C.c_void_p()

    def records(self) -> tuple[np.ndarray, np.ndarray]:
        n = lib().oracle_graph_size(self._h)
        keys = np.zeros(n, dtype=np.uint64)
        mult = np.zeros((n, 8), dtype=np.uint8)
        if n:
            lib().oracle_graph_get(self._h, keys.ctypes.data, mult.ctypes.data)
        return keys, mult

    def write_kmer_graph(self, path: str) -> None:
        lib().oracle_write_kmer_graph(self._h, self.k, str(path).encode())

    def write_node_lines(self, path: str) -> None:
        lib().oracle_write_node_lines(self._h, str(path).encode())

    def stats(self) -> list[int]:
        out = (C.c_int64 * 5)()
        lib().oracle_graph_stats(self._h, self.k, out)
        return list(out)


def build(text: bytes, k: int, cutoff: int, threads: int = 0, apply_cutoff: bool = True) -> OracleGraph:
    r = OracleReads()
    e = lib().oracle_parse_fasta(text, len(text), k, C.byref(r))
    if e:
        raise OracleError(e)
    try:
        h = lib().oracle_build(C.byref(r), k, cutoff, int(apply_cutoff), threads)
    finally:
        lib().oracle_reads_free(C.byref(r))
    if not h:
        raise OracleError(-5)
    return OracleGraph(h, k)


def records(text: bytes, k: int, cutoff: int, threads: int = 0) -> tuple[np.ndarray, np.ndarray]:
    return build(text, k, cutoff, threads).records()


def kmer_graph_neighbour(key: int, slot: int, k: int) -> int:
    return lib().oracle_kmer_graph_neighbour(key, slot, k)


def revcomp(x: int, k: int) -> int:
    return lib().oracle_revcomp(x, k)


MERGE_TIMING_REFERENCE = 0
MERGE_TIMING_IMMEDIATE = 1


def merge_tree_order(keys: np.ndarray, mult: np.ndarray, k: int) -> np.ndarray:
    """The node visiting order of the GPU merge (merge_oracle.c)."""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    mult = np.ascontiguousarray(mult, dtype=np.uint8).reshape(-1, 8)
    order = np.zeros(max(keys.size, 1), dtype=np.uint64)
    e = lib().oracle_merge_tree_order(k, keys.size, keys.ctypes.data, mult.ctypes.data, order.ctypes.data)
    if e:
        raise OracleError(e)
    return order[: keys.size]


def merge_text(keys: np.ndarray, mult: np.ndarray, k: int, order=None,
               timing: int = MERGE_TIMING_IMMEDIATE) -> bytes:
    """Merge semi-extended k-molecules visiting the nodes in `order` (node
    indices; default: the GPU merge's order) and return the -d file text
    (gathered node lines in visiting order, then '\n')."""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    mult = np.ascontiguousarray(mult, dtype=np.uint8).reshape(-1, 8)
    if order is None:
        order = merge_tree_order(keys, mult, k)
    order = np.ascontiguousarray(order, dtype=np.uint64)
    assert order.size == keys.size
    ptr, n, lines = C.c_void_p(), C.c_uint64(), C.c_uint64()
    e = lib().oracle_merge(k, keys.size, keys.ctypes.data, mult.ctypes.data, order.ctypes.data,
                           timing, C.byref(ptr), C.byref(n), C.byref(lines))
    if e:
        raise OracleError(e)
    try:
        return C.string_at(ptr.value, n.value) if n.value else b""
    finally:
        lib().oracle_free_text(ptr)


PRUNE_TIPS = 1
PRUNE_LOW_COVERAGE = 2


def prune_text(text: bytes, k: int, passes: int, order=None) -> tuple[bytes, int]:
    """masterTipsRemoval (passes & 1) then masterLowCoverageEdgeRemoval
    (passes & 2) on a merged graph given as gathered node lines, nodes visited
    in `order` (line indices; default file order). Returns the resulting
    gathered lines and the tips removed + arcs cut."""
    ptr, n, cnt = C.c_void_p(), C.c_uint64(), C.c_uint64()
    if order is not None:
        order = np.ascontiguousarray(order, dtype=np.uint64)
    e = lib().oracle_prune(k, text, len(text), order.ctypes.data if order is not None else None, passes,
                           C.byref(ptr), C.byref(n), C.byref(cnt))
    if e:
        raise OracleError(e)
    try:
        return (C.string_at(ptr.value, n.value) if n.value else b""), cnt.value
    finally:
        lib().oracle_free_text(ptr)


def simplify_text(text: bytes, k: int, order=None) -> tuple[bytes, int]:
    """masterSimplifyNodeGraph once over gathered lines, visiting them in
    `order` (line indices; default file order). Returns the resulting lines
    and the nodes merged away."""
    ptr, n, cnt = C.c_void_p(), C.c_uint64(), C.c_uint64()
    if order is not None:
        order = np.ascontiguousarray(order, dtype=np.uint64)
    e = lib().oracle_simplify_lines(k, text, len(text), order.ctypes.data if order is not None else None,
                                    C.byref(ptr), C.byref(n), C.byref(cnt))
    if e:
        raise OracleError(e)
    try:
        return (C.string_at(ptr.value, n.value) if n.value else b""), cnt.value
    finally:
        lib().oracle_free_text(ptr)


def lines_tree_order(text: bytes, k: int) -> np.ndarray:
    """The GPU's visiting order of masterSimplifyNodeGraph over these lines."""
    cap = max(text.count(b"\n"), 1)
    order = np.zeros(cap, dtype=np.uint64)
    n = C.c_uint64()
    e = lib().oracle_lines_tree_order(k, text, len(text), order.ctypes.data, cap, C.byref(n))
    if e:
        raise OracleError(e)
    return order[: n.value]


def run_reference_simplify(lines_path: str, k: int, cutoff: int, outdir: str,
                           timeout: float = 600) -> tuple[bytes, bytes]:
    """The reference's masterSimplifyNodeGraph on gathered lines: its graph
    before (node map order) and after the pass."""
    r = subprocess.run([str(HERE / "_ref" / "ref_simplify"), "-k", str(k), "-c", str(cutoff), "-i",
                        str(lines_path), "-o", str(outdir)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, timeout=timeout, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference simplify failed: %s" % r.stdout[-2000:])
    return Path(outdir, "before.txt").read_bytes(), Path(outdir, "after.txt").read_bytes()


CONTIG_LENGTH = 100  # sequence.h:15


def _rc_str(s: str) -> str:
    return s[::-1].translate(str.maketrans("ACGT", "TGCA"))


def contigs_of_lines(text: bytes, k: int) -> list[str]:
    """printContigs (graph.cpp:1139-1202) over gathered node lines: for every
    arc of at least Contig_Length - k bases whose node key is not smaller than
    the canonical id of the arc's last k bases, the node's k-mer (reverse
    complemented for slots 4-7) + the arc string. Sorted."""
    out = []
    for line in text.split(b"\n"):
        if not line.strip():
            continue
        head, rest = line.split(b" ", 1)
        key = int(head)
        arcs = [f.strip().decode() for f in rest.split(b"#")[:8]]
        kmer = "".join("ACGT"[(key >> (2 * (k - 1 - i))) & 3] for i in range(k))
        for i, a in enumerate(arcs):
            if not a or len(a) < CONTIG_LENGTH - k:
                continue
            d = (kmer if i < 4 else _rc_str(kmer)) + a
            last = d[-k:]
            canon = max(last, _rc_str(last))
            nid = 0
            for ch in canon:
                nid = nid * 4 + "ACGT".index(ch)
            if key < nid:
                continue
            out.append(d)
    return sorted(out)


def tips_last_order(text: bytes, k: int) -> np.ndarray:
    """The GPU's visiting order for the tip pass: every node that is not a tip
    (in key order), then the tips in key order; as line indices of `text`."""
    keys, tip = [], []
    for line in text.split(b"\n"):
        if not line.strip():
            continue
        head, rest = line.split(b" ", 1)
        arcs = [f.strip() for f in rest.split(b"#")[:8]]
        live = [a for a in arcs if a]
        keys.append(int(head))
        tip.append(len(live) == 1 and len(live[0]) < k)
    idx = sorted(range(len(keys)), key=lambda i: (tip[i], keys[i]))
    return np.array(idx, dtype=np.uint64)


def run_reference_prune(merged_path: str, k: int, cutoff: int, outdir: str,
                        timeout: float = 600) -> tuple[bytes, bytes, bytes]:
    """The reference's masterTipsRemoval and masterLowCoverageEdgeRemoval on a
    -d file: its graph (gathered lines, node map order) before, after the tip
    pass and after the low-coverage pass."""
    r = subprocess.run([str(HERE / "_ref" / "ref_prune"), "-k", str(k), "-c", str(cutoff), "-i",
                        str(merged_path), "-o", str(outdir)], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, timeout=timeout, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference prune failed: %s" % r.stdout[-2000:])
    return tuple(Path(outdir, f).read_bytes() for f in ("before.txt", "tips.txt", "lowcov.txt"))


def parse_node_lines(text: bytes) -> tuple[np.ndarray, np.ndarray]:
    """Keys and 8 multiplicities from node lines (graph.cpp:569 layout), in
    file order."""
    keys, mult = [], []
    for line in text.splitlines():
        if not line.strip():
            continue
        f = line.split()
        keys.append(int(f[0]))
        mult.append([int(x) for x in f[-8:]])
    return (np.array(keys, dtype=np.uint64),
            np.array(mult, dtype=np.uint8).reshape(-1, 8))


# ---- the reference itself (only where it was compiled from its sources) ----

def reference_available() -> bool:
    return REF_SWAP.exists() and REF_DUMP.exists() and REF_CONTIGS.exists() and (HERE / "_ref" / "ref_prune").exists() and (HERE / "_ref" / "ref_simplify").exists()


def run_reference(fasta_path: str, k: int, cutoff: int, outdir: str, timeout: float = 600) -> dict:
    """Run the reference's `swap -s` and its node dump on one FASTA.

    Returns the sorted kmerGraph.txt lines, the sorted node lines and the
    reference's stdout totals. outdir must not exist (the reference creates
    it, sequence.cpp:128-133)."""
    out = {}
    a, b = str(outdir) + "_s", str(outdir) + "_n"
    r = subprocess.run([str(REF_SWAP), "-k", str(k), "-c", str(cutoff), "-i", str(fasta_path),
                        "-o", a, "-s"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       timeout=timeout, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference swap failed: %s" % r.stdout[-2000:])
    out["kmer_graph"] = sorted(Path(a, "kmerGraph.txt").read_text().splitlines(),
                               key=lambda s: int(s.split()[0]))
    totals = {}
    for line in r.stdout.splitlines():
        if line.startswith("recv") and "=" in line:
            name, val = line.split("=")
            totals[name.strip()] = int(val)
    out["totals"] = totals
    r = subprocess.run([str(REF_DUMP), "-k", str(k), "-c", str(cutoff), "-i", str(fasta_path),
                        "-o", b], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       timeout=timeout, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference node dump failed: %s" % r.stdout[-2000:])
    out["nodes"] = sorted(Path(b, "nodes.txt").read_text().splitlines(),
                          key=lambda s: int(s.split()[0]))
    return out


def run_reference_merge(fasta_path: str, k: int, cutoff: int, outdir: str,
                        timeout: float = 600) -> tuple[bytes, bytes]:
    """The reference's node dump with -d: its nodes before the merge, in the
    order its merge visits them, and its contigGraph.txt after the merge
    (graph.cpp:1392-1566, 576-696). outdir must not exist."""
    r = subprocess.run([str(REF_DUMP), "-k", str(k), "-c", str(cutoff), "-i", str(fasta_path),
                        "-o", str(outdir), "-d"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       timeout=timeout, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference merge failed: %s" % r.stdout[-2000:])
    return Path(outdir, "nodes.txt").read_bytes(), Path(outdir, "contigGraph.txt").read_bytes()


def run_reference_contigs(merged_path: str, k: int, cutoff: int, outdir: str,
                          timeout: float = 600) -> tuple[list[str], list[str]]:
    """The reference's own rank-0 contig stage (graph.cpp:3629-3683) on a -d
    file: sorted sequences of noCEcontigs.fasta and CEContig.fasta."""
    r = subprocess.run([str(REF_CONTIGS), "-k", str(k), "-c", str(cutoff), "-i", str(merged_path),
                        "-o", str(outdir)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       timeout=timeout, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference contig stage failed: %s" % r.stdout[-2000:])
    return contig_sequences(Path(outdir, "noCEcontigs.fasta")), contig_sequences(Path(outdir, "CEContig.fasta"))


def contig_sequences(path) -> list[str]:
    """Sequences of a reference contig file: printContigs puts each on its
    header line after '>procN: ' (graph.cpp:1189), masterPrintContigs on the
    line after its header."""
    out = []
    for line in Path(path).read_text().splitlines():
        line = line.strip()
        if line.startswith(">proc"):
            out.append(line.split(": ", 1)[1])
        elif line and not line.startswith(">"):
            out.append(line)
    return sorted(out)


def cores() -> int:
    return os.cpu_count() or 1
