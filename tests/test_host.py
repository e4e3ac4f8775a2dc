"""Host-side parts of the library that need no GPU: FASTA framing and 2-bit
packing, the output writers, the C-ABI surface and the command line."""
import ctypes as C
import os
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
import swapgb
from common import golden, kat, kat_text, sha_lines, sorted_lines, synth_case_text

ROOT = Path(__file__).resolve().parent.parent


def unpack(reads: swapgb.Reads) -> np.ndarray:
    idx = np.arange(reads.n_bases, dtype=np.uint64)
    w = reads.packed[(idx >> np.uint64(4)).astype(np.int64)]
    sh = (np.uint64(30) - np.uint64(2) * (idx & np.uint64(15))).astype(np.uint32)
    return ((w >> sh) & 3).astype(np.uint8)


def same_framing(text: bytes, k: int) -> None:
    r = swapgb.reads_from_fasta(text, k)
    o = oracle.parse(text, k)
    assert r.n_reads == o["n_reads"] and r.n_bases == o["n_bases"]
    assert r.records == o["n_records"]
    assert np.array_equal(r.off, o["off"]) and np.array_equal(r.len, o["len"])
    assert np.array_equal(unpack(r), o["codes"])


@pytest.mark.parametrize("case", [c["name"] for c in golden()["kat"]])
def test_framing_matches_oracle_kat(case):
    same_framing(kat_text(case), kat(case)["k"])


def test_framing_large_parallel():
    # > 4 MiB per chunk: exercises the multi-threaded two-pass framing and the
    # words shared between chunks
    text = synth_case_text("c1_full")
    same_framing(text, 21)


def test_framing_leading_bytes_skipped():
    # bytes before the first '>' are skipped, as kmerGraph.cpp:113 does (the
    # reference then never finishes; this library does not hang on them)
    body = b">a\nACGTACGTACGTACGTACGTACGT\n>b\nTTTTGGGGCCCCAAAATTTTGGGG\n"
    r1 = swapgb.reads_from_fasta(b"junk\n\nmore junk\n" + body, 19)
    r2 = swapgb.reads_from_fasta(body, 19)
    assert np.array_equal(r1.packed, r2.packed) and np.array_equal(r1.len, r2.len)


@pytest.mark.parametrize("text,why", [
    (b">r1\nACGTACGTACGTACGTACGTAC", "last record without newline"),
    (b">r1\nACGTACGTACGTACGTACGTAC\n>r2\n", "header without sequence line"),
    (b"ACGTACGTACGTACGTACGTAC\n", "no record start"),
    (b">r1\nACGTACGT\x00ACGTACGTACGTAC\n", "NUL byte"),
    (b"", "empty input"),
])
def test_framing_rejects_what_the_reference_never_finishes(text, why):
    with pytest.raises(swapgb.SwgError) as e:
        swapgb.reads_from_fasta(text, 19)
    assert e.value.status == 1, why


def test_framing_bad_k():
    with pytest.raises(swapgb.SwgError):
        swapgb.reads_from_fasta(b">r\nACGT\n", 32)


@pytest.mark.parametrize("case", [c["name"] for c in golden()["kat"]])
def test_record_writers_match_reference(case, tmp_path):
    c = kat(case)
    keys, mult = oracle.records(kat_text(case), c["k"], c["c"])
    # writers take records in any order
    perm = np.random.default_rng(0).permutation(keys.size)
    swapgb.records_write_kmer_graph(keys[perm], mult[perm], c["k"], tmp_path / "kg.txt")
    swapgb.records_write_node_lines(keys[perm], mult[perm], tmp_path / "nodes.txt")
    assert sha_lines(sorted_lines(tmp_path / "kg.txt")) == c["kmer_graph_sha256"]
    assert sha_lines(sorted_lines(tmp_path / "nodes.txt")) == c["nodes_sha256"]
    # the library writes its lines already sorted by first token
    assert (tmp_path / "kg.txt").read_text().splitlines() == sorted_lines(tmp_path / "kg.txt")


def test_abi_exports_every_declared_symbol():
    header = (ROOT / "include" / "swapgb.h").read_text()
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)  # declarations only
    declared = set(re.findall(r"\b(swg_\w+)\s*\(", header))
    out = subprocess.run(["nm", "-D", "--defined-only", str(swapgb.LIB_PATH)],
                         stdout=subprocess.PIPE, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert declared, "no declarations parsed"
    assert declared <= exported, sorted(declared - exported)
    lib = swapgb.lib()
    for name in declared:
        assert hasattr(lib, name)


C_CALLER = r"""
#include <stdio.h>
#include <stdlib.h>
#include "swapgb.h"
int main(int argc, char **argv) {
    swg_reads *reads = NULL;
    if (argc < 2 || swg_reads_from_fasta_file(argv[1], 31, &reads) != SWG_OK) return 1;
    const uint32_t *packed; const uint64_t *off; const uint32_t *len;
    uint64_t n_words, n_reads, n_bases;
    swg_reads_view(reads, &packed, &n_words, &off, &len, &n_reads, &n_bases);
    swg_opts o = {0};
    o.k = 31; o.cutoff = 5;
    swg_graph *g = NULL;
    swg_status st = swg_build(&o, packed, n_words, off, len, n_reads, &g);
    swg_reads_free(reads);
    if (st != SWG_OK) { printf("%s\n", swg_last_error()); return 1; }
    uint64_t n = 0, bytes = 0, removed = 0, merged = 0, cut = 0;
    swg_graph_size(g, &n);
    uint64_t *keys = malloc(8 * n); uint8_t *mult = malloc(8 * n);
    swg_graph_copy_out(g, keys, mult, n, 0, &n);
    swg_graph_merge(g);
    swg_graph_copy_merged(g, NULL, 0, &bytes);
    swg_graph_remove_tips(g, &removed); swg_graph_simplify(g, &merged);
    swg_graph_remove_low_coverage(g, &cut); swg_graph_simplify(g, &merged);
    swg_merge_info mi; swg_graph_merge_info(g, &mi);
    swg_graph_write_merged(g, "contigGraph.txt");
    swg_graph_free(g); free(keys); free(mult);
    return 0;
}
"""


def test_header_is_plain_c_and_links(tmp_path):
    """A C caller (no C++, no CUDA headers) compiles against include/swapgb.h
    with warnings as errors and links against libswapgb.so."""
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I" + str(ROOT / "include"),
                        str(src), "-L" + str(swapgb.LIB_PATH.parent), "-lswapgb",
                        "-Wl,-rpath," + str(swapgb.LIB_PATH.parent), "-o", str(tmp_path / "caller")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


STRUCTS = [("swg_opts", swapgb.Opts), ("swg_build_info", swapgb.BuildInfo), ("swg_merge_info", swapgb.MergeInfo),
           ("swg_sample", swapgb.Sample), ("swg_server_opts", swapgb.ServerOpts),
           ("swg_server_stats", swapgb.ServerStats), ("swg_tuning", swapgb.Tuning)]


def test_ctypes_mirrors_match_the_header(tmp_path):
    """Every struct swapgb.py mirrors has the header's size and field offsets
    (a C program compiled against include/swapgb.h prints them)."""
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "swapgb.h"', "int main(void) {"]
    for cname, py in STRUCTS:
        lines.append('    printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in py._fields_:
            lines.append('    printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I" + str(ROOT / "include"), str(src), "-o", str(exe)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    got = {}
    for line in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True, check=True).stdout.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, py in STRUCTS:
        assert got[(cname, "size")] == C.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_host_code_under_address_and_undefined_sanitizers(tmp_path):
    """The host FASTA framing/packing (multi-threaded) and the text writers,
    compiled with -fsanitize=address,undefined, over the golden known-answer
    inputs, malformed inputs and random records: no sanitizer report."""
    import shutil
    if not shutil.which("g++"):
        pytest.skip("no g++")
    cuda_inc = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
    csrc = ROOT / "swap-assembler_gb300" / "csrc"
    exe = tmp_path / "host_sanitize"
    r = subprocess.run(["g++", "-std=c++17", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-g",
                        "-O1", "-I" + str(ROOT / "include"), "-I" + str(csrc), "-I" + cuda_inc,
                        str(csrc / "reads.cpp"), str(csrc / "writers.cpp"),
                        str(ROOT / "tests" / "sanitize" / "host_sanitize.cpp"), "-lpthread", "-o", str(exe)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, stdin=subprocess.DEVNULL)
    if r.returncode != 0 and "sanitize" in r.stdout:
        pytest.skip("sanitizer runtime not available: " + r.stdout[-300:])
    assert r.returncode == 0, r.stdout
    inputs = sorted(str(p) for p in (ROOT / "tests" / "golden").glob("*.fa"))
    env = dict(os.environ, SWG_SANITIZE_OUT=str(tmp_path))
    r = subprocess.run([str(exe), *inputs], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       env=env, stdin=subprocess.DEVNULL, timeout=600)
    assert r.returncode == 0 and "clean" in r.stdout, r.stdout[-3000:]


def test_status_strings():
    lib = swapgb.lib()
    for s in range(11):
        assert lib.swg_status_string(s)
    assert lib.swg_version().startswith(b"swapgb")


def test_cli_argument_checks(tmp_path):
    swap = str(swapgb.SWAP_BIN)
    r = subprocess.run([swap, "-k", "20", "-i", "x.fa", "-o", str(tmp_path / "o")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 2 and "odd number" in r.stdout
    r = subprocess.run([swap, "-k", "33", "-i", "x.fa", "-o", str(tmp_path / "o")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 2
    r = subprocess.run([swap, "-k", "21"], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 2 and "Usage" in r.stdout
    (tmp_path / "exists").mkdir()
    r = subprocess.run([swap, "-i", "x.fa", "-o", str(tmp_path / "exists")],
                       stdout=subprocess.PIPE, text=True)
    assert r.returncode == 1 and "Creating directory" in r.stdout
    r = subprocess.run([swap, "-v"], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0 and "version" in r.stdout


def test_synthetic_generator_is_deterministic():
    a = swapgb.synth_fasta(seed=5, genome_len=50000, n_reads=5000, read_len=150, sub_rate=0.01,
                           indel_rate=0.001, repeat_frac=0.05, tandem_frac=0.02, threads=1)
    b = swapgb.synth_fasta(seed=5, genome_len=50000, n_reads=5000, read_len=150, sub_rate=0.01,
                           indel_rate=0.001, repeat_frac=0.05, tandem_frac=0.02, threads=5)
    assert a == b
    lines = a.split(b"\n")
    assert lines[0] == b">r0" and all(len(x) == 150 for x in lines[1:-1:2])


def test_autotune_cache_lookup(tmp_path):
    cache = tmp_path / "tune.jsonl"
    opts = swapgb.Opts(k=31, cutoff=5)
    assert not swapgb.autotune_apply(cache, 31, 100, opts)  # no file yet
    cache.write_text(
        '{"k": 31, "band": 1, "load": 0.700, "algorithm": 1, "read_order": 0, "ms": 9.1}\n'
        '{"k": 27, "band": 2, "load": 0.500, "algorithm": 2, "read_order": 0, "ms": 1.0}\n'
        '{"k": 31, "band": 1, "load": 0.800, "algorithm": 1, "read_order": 1, "ms": 8.0}\n')
    assert swapgb.autotune_apply(cache, 31, 100, opts)  # 100 bp -> band 1; last entry wins
    assert abs(opts.load_factor - 0.8) < 1e-9 and opts.algorithm == 1 and opts.read_order == 1
    assert swapgb.autotune_apply(cache, 27, 150, opts) and opts.algorithm == 2
    assert not swapgb.autotune_apply(cache, 27, 250, opts)
    # entries with the bucketed knobs fill them too; the older form leaves them 0
    with open(cache, "a") as f:
        f.write('{"k": 27, "band": 3, "load": 0.600, "algorithm": 3, "read_order": 0, "ms": 2.5, '
                '"bucket_records": 8192, "part_bits": 9, "scatter_shape": 2}\n')
    assert swapgb.autotune_apply(cache, 27, 250, opts)
    assert (opts.algorithm, opts.bucket_records, opts.part_bits, opts.scatter_shape) == (3, 8192, 9, 2)
    assert swapgb.autotune_apply(cache, 27, 150, opts)
    assert (opts.bucket_records, opts.part_bits, opts.scatter_shape) == (0, 0, 0)
