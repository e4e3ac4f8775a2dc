"""ctypes binding of the GB300 k-mer graph builder (C ABI in include/swapgb.h).

This is a thin host-side mirror of the library: it loads the in-tree
libswapgb.so (built by build.py) and raises if it is missing. There is no
Python or CPU implementation of the build behind it.

    reads = reads_from_fasta(text, k=31)
    g = Graph()
    g.build(Opts(k=31, cutoff=5), reads.packed, reads.off, reads.len)
    keys, mult = g.copy_out(sorted=True)   # uint64[n], uint8[n, 8]
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libswapgb.so"
SYNTH_PATH = PKG / "libswgsynth.so"
SWAP_BIN = PKG / "bin" / "swap"

STATUS = {
    0: "SWG_OK", 1: "SWG_ERR_BAD_INPUT", 2: "SWG_ERR_TABLE_FULL", 3: "SWG_ERR_OOM",
    4: "SWG_ERR_ADMISSION", 5: "SWG_ERR_TIMEOUT", 6: "SWG_ERR_CUDA", 7: "SWG_ERR_NO_DEVICE",
    8: "SWG_ERR_BAD_STATE", 9: "SWG_ERR_IO", 10: "SWG_ERR_NOT_READY",
}


class SwgError(RuntimeError):
    def __init__(self, status: int, what: str, msg: str):
        super().__init__("%s: %s (%s)" % (what, STATUS.get(status, status), msg))
        self.status = status


ALGO_DEFAULT, ALGO_DIRECT, ALGO_PARTITIONED, ALGO_BUCKETED = 0, 1, 2, 3
ORDER_INPUT, ORDER_MINIMIZER = 0, 1


class Opts(C.Structure):
    _fields_ = [("k", C.c_int), ("cutoff", C.c_int), ("load_factor", C.c_double),
                ("expected_distinct", C.c_uint64), ("stream", C.c_void_p),
                ("algorithm", C.c_int), ("read_order", C.c_int),
                ("bucket_records", C.c_uint32), ("part_bits", C.c_int), ("scatter_shape", C.c_int)]

    def __init__(self, k: int = 23, cutoff: int = 5, load_factor: float = 0.0,
                 expected_distinct: int = 0, stream: int | None = None, algorithm: int = 0,
                 read_order: int = 0, bucket_records: int = 0, part_bits: int = 0,
                 scatter_shape: int = 0):
        super().__init__(k, cutoff, load_factor, expected_distinct, stream, algorithm,
                         read_order, bucket_records, part_bits, scatter_shape)


class BuildInfo(C.Structure):
    _fields_ = [("algorithm", C.c_int), ("launches", C.c_int), ("occurrences", C.c_uint64),
                ("distinct", C.c_uint64), ("survivors", C.c_uint64),
                ("table_entries", C.c_uint64), ("partitions", C.c_uint32),
                ("slots", C.c_uint32), ("waves", C.c_uint32), ("retries", C.c_uint32),
                ("estimate", C.c_double), ("ms", C.c_float * 5), ("bucket_table", C.c_uint32)]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "ms"}
        d["ms"] = list(self.ms)
        return d


class MergeInfo(C.Structure):
    _fields_ = [("nodes", C.c_uint64), ("chains", C.c_uint64), ("cycles", C.c_uint64),
                ("text_bytes", C.c_uint64), ("ms", C.c_float), ("launches", C.c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Sample(C.Structure):
    _fields_ = [("packed", C.c_void_p), ("n_words", C.c_uint64), ("read_off", C.c_void_p),
                ("read_len", C.c_void_p), ("n_reads", C.c_uint64), ("k", C.c_int),
                ("cutoff", C.c_int)]


class ServerOpts(C.Structure):
    _fields_ = [("memory_budget", C.c_uint64), ("workers", C.c_uint32), ("max_batch", C.c_uint32),
                ("load_factor", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "failed", "rejected", "batches",
                                          "max_batch_requests", "queued", "bytes_reserved",
                                          "bytes_resident")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3

class Tuning(C.Structure):
    _fields_ = [("load_factor", C.c_double), ("algorithm", C.c_int), ("read_order", C.c_int),
                ("ms", C.c_float), ("bucket_records", C.c_uint32), ("part_bits", C.c_int),
                ("scatter_shape", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    """The loaded libswapgb.so; raises if the native library has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError("native library %s is missing: run build()" % LIB_PATH)
        L = C.CDLL(str(LIB_PATH))
        P, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
        pu64 = C.POINTER(C.c_uint64)
        sigs = {
            "swg_status_string": (C.c_char_p, [i32]),
            "swg_last_error": (C.c_char_p, []),
            "swg_version": (C.c_char_p, []),
            "swg_reads_from_fasta": (i32, [C.c_char_p, u64, i32, C.POINTER(P)]),
            "swg_reads_from_fasta_file": (i32, [C.c_char_p, i32, C.POINTER(P)]),
            "swg_reads_view": (i32, [P, C.POINTER(P), pu64, C.POINTER(P), C.POINTER(P), pu64, pu64]),
            "swg_reads_records": (u64, [P]),
            "swg_reads_free": (None, [P]),
            "swg_graph_create": (i32, [C.POINTER(P)]),
            "swg_graph_free": (None, [P]),
            "swg_graph_build": (i32, [P, C.POINTER(Opts), P, u64, P, P, u64]),
            "swg_graph_build_device": (i32, [P, C.POINTER(Opts), P, u64, P, P, u64]),
            "swg_build": (i32, [C.POINTER(Opts), P, u64, P, P, u64, C.POINTER(P)]),
            "swg_build_fasta": (i32, [C.POINTER(Opts), C.c_char_p, u64, C.POINTER(P)]),
            "swg_graph_build_fasta": (i32, [P, C.POINTER(Opts), P, u64]),
            "swg_graph_build_fasta_file": (i32, [P, C.POINTER(Opts), C.c_char_p]),
            "swg_graph_build_fasta_to_host": (i32, [P, C.POINTER(Opts), P, u64, P, P, u64, pu64]),
            "swg_graph_size": (i32, [P, pu64]),
            "swg_graph_distinct": (i32, [P, pu64]),
            "swg_graph_device_view": (i32, [P, C.POINTER(P), C.POINTER(P), pu64]),
            "swg_graph_copy_out": (i32, [P, P, P, u64, i32, pu64]),
            "swg_graph_stats": (i32, [P, C.POINTER(C.c_int64)]),
            "swg_graph_write_kmer_graph": (i32, [P, C.c_char_p]),
            "swg_graph_write_node_lines": (i32, [P, C.c_char_p]),
            "swg_graph_merge": (i32, [P]),
            "swg_graph_merge_in_order": (i32, [P, P, u64]),
            "swg_graph_merge_info": (i32, [P, C.POINTER(MergeInfo)]),
            "swg_graph_write_merged": (i32, [P, C.c_char_p]),
            "swg_graph_copy_merged": (i32, [P, P, u64, pu64]),
            "swg_graph_remove_tips": (i32, [P, pu64]),
            "swg_graph_remove_low_coverage": (i32, [P, pu64]),
            "swg_graph_simplify": (i32, [P, pu64]),
            "swg_graph_write_contigs": (i32, [P, C.c_char_p, pu64]),
            "swg_records_write_kmer_graph": (i32, [P, P, u64, i32, C.c_char_p]),
            "swg_records_write_node_lines": (i32, [P, P, u64, C.c_char_p]),
            "swg_graph_last_timings": (i32, [P, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
            "swg_graph_build_info": (i32, [P, C.POINTER(BuildInfo)]),
            "swg_probe_random_access": (i32, [i32, u64, u64, P, C.POINTER(C.c_double)]),
            "swg_probe_shared_atomics": (i32, [i32, u64, P, C.POINTER(C.c_double)]),
            "swg_batch_build": (i32, [P, C.POINTER(Opts), C.POINTER(Sample), C.c_uint32]),
            "swg_batch_samples": (i32, [P, C.POINTER(C.c_uint32)]),
            "swg_batch_sample_info": (i32, [P, C.c_uint32, pu64, pu64, pu64]),
            "swg_batch_device_view": (i32, [P, C.c_uint32, C.POINTER(P), C.POINTER(P), pu64]),
            "swg_batch_copy_out": (i32, [P, C.c_uint32, P, P, u64, i32, pu64]),
            "swg_server_create": (i32, [C.POINTER(ServerOpts), C.POINTER(P)]),
            "swg_server_submit": (i32, [P, C.POINTER(Sample), pu64]),
            "swg_server_poll": (i32, [P, u64, C.POINTER(i32), C.POINTER(C.c_double)]),
            "swg_server_wait": (i32, [P, u64, C.c_double]),
            "swg_server_result_info": (i32, [P, u64, pu64, pu64]),
            "swg_server_fetch": (i32, [P, u64, P, P, u64, i32, pu64]),
            "swg_server_release": (i32, [P, u64]),
            "swg_server_get_stats": (i32, [P, C.POINTER(ServerStats)]),
            "swg_server_free": (None, [P]),
            "swg_autotune": (i32, [C.POINTER(Opts), P, u64, P, P, u64, C.c_uint32, C.c_char_p,
                                   C.POINTER(Tuning)]),
            "swg_autotune_apply": (i32, [C.c_char_p, i32, C.c_uint32, C.POINTER(Opts)]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status != 0:
        raise SwgError(status, what, lib().swg_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a.size else 0


class Reads:
    """Packed reads on the host (swg_reads), with numpy views of its arrays."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        p, off, ln = C.c_void_p(), C.c_void_p(), C.c_void_p()
        nw, nr, nb = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().swg_reads_view(self._h, C.byref(p), C.byref(nw), C.byref(off), C.byref(ln),
                                    C.byref(nr), C.byref(nb)), "swg_reads_view")
        self.n_words, self.n_reads, self.n_bases = nw.value, nr.value, nb.value
        self.records = lib().swg_reads_records(self._h)
        self.packed = _view(p.value, nw.value, np.uint32)
        self.off = _view(off.value, nr.value, np.uint64)
        self.len = _view(ln.value, nr.value, np.uint32)

    def close(self) -> None:
        if self._h:
            lib().swg_reads_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _view(addr: int | None, n: int, dtype) -> np.ndarray:
    if not n or not addr:
        return np.zeros(0, dtype=dtype)
    buf = (C.c_char * (n * np.dtype(dtype).itemsize)).from_address(addr)
    return np.frombuffer(buf, dtype=dtype, count=n)


def reads_from_fasta(text: bytes, k: int) -> Reads:
    h = C.c_void_p()
    _check(lib().swg_reads_from_fasta(text, len(text), k, C.byref(h)), "swg_reads_from_fasta")
    return Reads(h.value)


def reads_from_fasta_file(path: str, k: int) -> Reads:
    h = C.c_void_p()
    _check(lib().swg_reads_from_fasta_file(str(path).encode(), k, C.byref(h)),
           "swg_reads_from_fasta_file")
    return Reads(h.value)


class Graph:
    """A device-resident filtered k-mer graph (swg_graph) and its workspace."""

    def __init__(self):
        h = C.c_void_p()
        _check(lib().swg_graph_create(C.byref(h)), "swg_graph_create")
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().swg_graph_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, opts: Opts, packed: np.ndarray, off: np.ndarray, ln: np.ndarray) -> "Graph":
        packed = np.ascontiguousarray(packed, dtype=np.uint32)
        off = np.ascontiguousarray(off, dtype=np.uint64)
        ln = np.ascontiguousarray(ln, dtype=np.uint32)
        _check(lib().swg_graph_build(self._h, C.byref(opts), _ptr(packed), packed.size, _ptr(off),
                                     _ptr(ln), off.size), "swg_graph_build")
        return self

    def build_reads(self, opts: Opts, reads: Reads) -> "Graph":
        return self.build(opts, reads.packed, reads.off, reads.len)

    def build_device(self, opts: Opts, d_packed: int, n_words: int, d_off: int, d_len: int,
                     n_reads: int) -> "Graph":
        _check(lib().swg_graph_build_device(self._h, C.byref(opts), d_packed, n_words, d_off,
                                            d_len, n_reads), "swg_graph_build_device")
        return self

    def size(self) -> int:
        n = C.c_uint64()
        _check(lib().swg_graph_size(self._h, C.byref(n)), "swg_graph_size")
        return n.value

    def distinct(self) -> int:
        n = C.c_uint64()
        _check(lib().swg_graph_distinct(self._h, C.byref(n)), "swg_graph_distinct")
        return n.value

    def device_view(self) -> tuple[int, int, int]:
        k, m, n = C.c_void_p(), C.c_void_p(), C.c_uint64()
        _check(lib().swg_graph_device_view(self._h, C.byref(k), C.byref(m), C.byref(n)),
               "swg_graph_device_view")
        return k.value or 0, m.value or 0, n.value

    def copy_out(self, sorted: bool = True) -> tuple[np.ndarray, np.ndarray]:
        n = self.size()
        keys = np.zeros(n, dtype=np.uint64)
        mult = np.zeros((n, 8), dtype=np.uint8)
        got = C.c_uint64()
        _check(lib().swg_graph_copy_out(self._h, _ptr(keys), _ptr(mult), n, int(sorted),
                                        C.byref(got)), "swg_graph_copy_out")
        return keys, mult

    def stats(self) -> list[int]:
        out = (C.c_int64 * 5)()
        _check(lib().swg_graph_stats(self._h, out), "swg_graph_stats")
        return list(out)

    def write_kmer_graph(self, path: str) -> None:
        _check(lib().swg_graph_write_kmer_graph(self._h, str(path).encode()),
               "swg_graph_write_kmer_graph")

    def write_node_lines(self, path: str) -> None:
        _check(lib().swg_graph_write_node_lines(self._h, str(path).encode()),
               "swg_graph_write_node_lines")

    def merge(self) -> "Graph":
        """Merge the semi-extended k-molecules of the built graph on the device."""
        _check(lib().swg_graph_merge(self._h), "swg_graph_merge")
        return self

    def merge_in_order(self, order_keys: np.ndarray) -> "Graph":
        """The merge with the nodes visited in the given order (every key of the
        built graph once)."""
        ok = np.ascontiguousarray(order_keys, dtype=np.uint64)
        _check(lib().swg_graph_merge_in_order(self._h, _ptr(ok), ok.size), "swg_graph_merge_in_order")
        return self

    def merge_info(self) -> dict:
        info = MergeInfo()
        _check(lib().swg_graph_merge_info(self._h, C.byref(info)), "swg_graph_merge_info")
        return info.as_dict()

    def merged_text(self) -> bytes:
        """The merged graph as the -d file's bytes (contigGraph.txt)."""
        n = C.c_uint64()
        lib().swg_graph_copy_merged(self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(max(n.value, 1))
        _check(lib().swg_graph_copy_merged(self._h, C.addressof(buf), n.value, C.byref(n)),
               "swg_graph_copy_merged")
        return buf.raw[: n.value]

    def remove_tips(self) -> int:
        """masterTipsRemoval on the merged graph; returns the nodes deleted."""
        n = C.c_uint64()
        _check(lib().swg_graph_remove_tips(self._h, C.byref(n)), "swg_graph_remove_tips")
        return n.value

    def remove_low_coverage(self) -> int:
        """masterLowCoverageEdgeRemoval on the merged graph; returns the arcs cut."""
        n = C.c_uint64()
        _check(lib().swg_graph_remove_low_coverage(self._h, C.byref(n)), "swg_graph_remove_low_coverage")
        return n.value

    def simplify(self) -> int:
        """masterSimplifyNodeGraph on the merged graph; returns the nodes merged away."""
        n = C.c_uint64()
        _check(lib().swg_graph_simplify(self._h, C.byref(n)), "swg_graph_simplify")
        return n.value

    def write_contigs(self, path: str) -> int:
        """printContigs of the merged graph into `path`; returns the contigs written."""
        n = C.c_uint64()
        _check(lib().swg_graph_write_contigs(self._h, str(path).encode(), C.byref(n)), "swg_graph_write_contigs")
        return n.value

    def write_merged(self, path: str) -> None:
        _check(lib().swg_graph_write_merged(self._h, str(path).encode()), "swg_graph_write_merged")

    def build_fasta(self, opts: Opts, text) -> "Graph":
        """Frame and pack the FASTA on the device, then build. `text` is bytes
        or a host buffer address with its length as (addr, n)."""
        if isinstance(text, tuple):
            addr, n = text
        else:
            buf = C.create_string_buffer(text, len(text))
            addr, n = C.addressof(buf), len(text)
        _check(lib().swg_graph_build_fasta(self._h, C.byref(opts), addr, n), "swg_graph_build_fasta")
        return self

    def build_fasta_file(self, opts: Opts, path: str) -> "Graph":
        """Build from a FASTA file (read into a pinned buffer, framed on the device)."""
        _check(lib().swg_graph_build_fasta_file(self._h, C.byref(opts), str(path).encode()),
               "swg_graph_build_fasta_file")
        return self

    def build_batch(self, opts: Opts, samples: list) -> "Graph":
        """samples: list of (Reads, k, cutoff). Each sample gets its own result."""
        arr = (Sample * len(samples))()
        for i, (r, k, c) in enumerate(samples):
            arr[i] = Sample(_ptr(r.packed), r.n_words, _ptr(r.off), _ptr(r.len), r.n_reads, k, c)
        self._batch_keepalive = samples
        _check(lib().swg_batch_build(self._h, C.byref(opts), arr, len(samples)), "swg_batch_build")
        return self

    def batch_size(self) -> int:
        n = C.c_uint32()
        _check(lib().swg_batch_samples(self._h, C.byref(n)), "swg_batch_samples")
        return n.value

    def batch_info(self, s: int) -> tuple[int, int, int]:
        o, d, v = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().swg_batch_sample_info(self._h, s, C.byref(o), C.byref(d), C.byref(v)),
               "swg_batch_sample_info")
        return o.value, d.value, v.value

    def batch_copy_out(self, s: int, sorted: bool = True) -> tuple[np.ndarray, np.ndarray]:
        n = self.batch_info(s)[2]
        keys = np.zeros(n, dtype=np.uint64)
        mult = np.zeros((n, 8), dtype=np.uint8)
        got = C.c_uint64()
        _check(lib().swg_batch_copy_out(self._h, s, _ptr(keys), _ptr(mult), n, int(sorted),
                                        C.byref(got)), "swg_batch_copy_out")
        return keys, mult

    def info(self) -> dict:
        bi = BuildInfo()
        _check(lib().swg_graph_build_info(self._h, C.byref(bi)), "swg_graph_build_info")
        return bi.as_dict()

    def timings(self) -> tuple[list[float], int]:
        ms = (C.c_float * 5)()
        n = C.c_int()
        _check(lib().swg_graph_last_timings(self._h, ms, C.byref(n)), "swg_graph_last_timings")
        return list(ms), n.value


def build_fasta(opts: Opts, text: bytes) -> Graph:
    g = Graph.__new__(Graph)
    h = C.c_void_p()
    _check(lib().swg_build_fasta(C.byref(opts), text, len(text), C.byref(h)), "swg_build_fasta")
    g._h = h
    return g


def records_write_kmer_graph(keys: np.ndarray, mult: np.ndarray, k: int, path: str) -> None:
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    mult = np.ascontiguousarray(mult, dtype=np.uint8).reshape(-1, 8)
    _check(lib().swg_records_write_kmer_graph(_ptr(keys), _ptr(mult), keys.size, k,
                                              str(path).encode()), "swg_records_write_kmer_graph")


def records_write_node_lines(keys: np.ndarray, mult: np.ndarray, path: str) -> None:
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    mult = np.ascontiguousarray(mult, dtype=np.uint8).reshape(-1, 8)
    _check(lib().swg_records_write_node_lines(_ptr(keys), _ptr(mult), keys.size,
                                              str(path).encode()), "swg_records_write_node_lines")


PROBE_KINDS = {"red_add_u32": 0, "atom_add_u64": 1, "cas128": 2, "load16": 3, "load16_cas128": 4,
               "load16_x4": 5, "load16_cas128_x2": 6}


def probe_shared_atomics(kind: str, n_ops: int, stream: int | None = None) -> float:
    """Lane operations per second of random shared-memory atomics (whole GPU)."""
    out = C.c_double()
    _check(lib().swg_probe_shared_atomics({"add_u32": 0, "cas_u64": 1}[kind], n_ops, stream, C.byref(out)),
           "swg_probe_shared_atomics")
    return out.value


def probe_random_access(kind: str, table_bytes: int, n_ops: int, stream: int | None = None) -> float:
    """Random-access operations per second on this GPU (device time)."""
    out = C.c_double()
    _check(lib().swg_probe_random_access(PROBE_KINDS[kind], table_bytes, n_ops, stream,
                                         C.byref(out)), "swg_probe_random_access")
    return out.value


# ---- synthetic reads ------------------------------------------------------

class SynthParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("genome_len", C.c_uint64), ("gc", C.c_double),
                ("repeat_frac", C.c_double), ("repeat_unit_min", C.c_uint32),
                ("repeat_unit_max", C.c_uint32), ("repeat_copies_min", C.c_uint32),
                ("repeat_copies_max", C.c_uint32), ("repeat_divergence", C.c_double),
                ("tandem_frac", C.c_double), ("tandem_unit_min", C.c_uint32),
                ("tandem_unit_max", C.c_uint32), ("tandem_len_min", C.c_uint32),
                ("tandem_len_max", C.c_uint32), ("n_reads", C.c_uint64), ("read_len", C.c_uint32),
                ("sub_rate", C.c_double), ("indel_rate", C.c_double), ("threads", C.c_int)]


_synth = None


def _synth_lib() -> C.CDLL:
    global _synth
    if _synth is None:
        if not SYNTH_PATH.exists():
            raise RuntimeError("%s is missing: run build()" % SYNTH_PATH)
        L = C.CDLL(str(SYNTH_PATH))
        L.swg_synth_defaults.argtypes = [C.POINTER(SynthParams)]
        L.swg_synth_defaults.restype = None
        L.swg_synth_fasta.argtypes = [C.POINTER(SynthParams), C.POINTER(C.c_void_p)]
        L.swg_synth_fasta.restype = C.c_int64
        L.swg_synth_fasta_file.argtypes = [C.POINTER(SynthParams), C.c_char_p]
        L.swg_synth_fasta_file.restype = C.c_int64
        L.swg_synth_free.argtypes = [C.c_void_p]
        L.swg_synth_free.restype = None
        _synth = L
    return _synth


def synth_params(**kw) -> SynthParams:
    p = SynthParams()
    _synth_lib().swg_synth_defaults(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def synth_fasta(**kw) -> bytes:
    """Seeded synthetic FASTA (see csrc/synth.h for the parameters)."""
    p = synth_params(**kw)
    buf = C.c_void_p()
    n = _synth_lib().swg_synth_fasta(C.byref(p), C.byref(buf))
    if n < 0:
        raise RuntimeError("synthetic read generation failed")
    try:  # (string_at takes a C int size: no good past 2 GiB)
        return bytes((C.c_ubyte * n).from_address(buf.value)) if n else b""
    finally:
        _synth_lib().swg_synth_free(buf)


def batch_workload_specs(n: int = 256, seed: int = 4) -> list[dict]:
    """Generator parameters of the batched workload's samples: genome sizes
    log-uniform 50 kbp-2 Mbp, read length from {75, 100, 150, 250}, coverage
    uniform 10-60x, substitutions uniform 0.1-1% (built with k=27, c=3)."""
    import math
    import random
    rng = random.Random(seed)
    out = []
    for i in range(n):
        g = int(math.exp(rng.uniform(math.log(50_000), math.log(2_000_000))))
        L = rng.choice([75, 100, 150, 250])
        cov = rng.uniform(10, 60)
        out.append(dict(seed=10_000 + i, genome_len=g, n_reads=int(cov * g / L), read_len=L,
                        sub_rate=rng.uniform(0.001, 0.01)))
    return out


def synth_fasta_file(path: str, **kw) -> int:
    p = synth_params(**kw)
    n = _synth_lib().swg_synth_fasta_file(C.byref(p), str(path).encode())
    if n < 0:
        raise RuntimeError("synthetic read generation failed")
    return n


class Server:
    """Request server (continuous batching); results stay on the device until
    fetched or released."""

    def __init__(self, memory_budget: int = 0, workers: int = 0, max_batch: int = 0,
                 load_factor: float = 0.0):
        h = C.c_void_p()
        o = ServerOpts(memory_budget, workers, max_batch, load_factor)
        _check(lib().swg_server_create(C.byref(o), C.byref(h)), "swg_server_create")
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().swg_server_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, reads: Reads, k: int, cutoff: int) -> int:
        smp = Sample(_ptr(reads.packed), reads.n_words, _ptr(reads.off), _ptr(reads.len),
                     reads.n_reads, k, cutoff)
        t = C.c_uint64()
        _check(lib().swg_server_submit(self._h, C.byref(smp), C.byref(t)), "swg_server_submit")
        return t.value

    def poll(self, ticket: int) -> tuple[int, float]:
        st, lat = C.c_int(), C.c_double()
        _check(lib().swg_server_poll(self._h, ticket, C.byref(st), C.byref(lat)), "swg_server_poll")
        return st.value, lat.value

    def wait(self, ticket: int, timeout_s: float = 60.0) -> None:
        _check(lib().swg_server_wait(self._h, ticket, timeout_s), "swg_server_wait")

    def fetch(self, ticket: int, sorted: bool = True) -> tuple[np.ndarray, np.ndarray]:
        n, d = C.c_uint64(), C.c_uint64()
        _check(lib().swg_server_result_info(self._h, ticket, C.byref(n), C.byref(d)),
               "swg_server_result_info")
        keys = np.zeros(n.value, dtype=np.uint64)
        mult = np.zeros((n.value, 8), dtype=np.uint8)
        got = C.c_uint64()
        _check(lib().swg_server_fetch(self._h, ticket, _ptr(keys), _ptr(mult), n.value, int(sorted),
                                      C.byref(got)), "swg_server_fetch")
        return keys, mult

    def release(self, ticket: int) -> None:
        _check(lib().swg_server_release(self._h, ticket), "swg_server_release")

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().swg_server_get_stats(self._h, C.byref(st)), "swg_server_get_stats")
        return st.as_dict()


def autotune(opts: Opts, d_packed: int, n_words: int, d_off: int, d_len: int, n_reads: int,
             read_len: int, cache_path: str) -> dict:
    t = Tuning()
    _check(lib().swg_autotune(C.byref(opts), d_packed, n_words, d_off, d_len, n_reads, read_len,
                              str(cache_path).encode(), C.byref(t)), "swg_autotune")
    return {"load_factor": t.load_factor, "algorithm": t.algorithm, "read_order": t.read_order,
            "ms": t.ms, "bucket_records": t.bucket_records, "part_bits": t.part_bits,
            "scatter_shape": t.scatter_shape}


def autotune_apply(cache_path: str, k: int, read_len: int, opts: Opts) -> bool:
    """Fill opts from the cache; False when the cache has no entry."""
    st = lib().swg_autotune_apply(str(cache_path).encode(), k, read_len, C.byref(opts))
    if st == 10:
        return False
    _check(st, "swg_autotune_apply")
    return True
