"""swg_build_device_noalloc: the build for callers that cannot let the library
allocate device memory (their GPU memory belongs to another allocator or a
fixed budget, or a mid-run cudaMalloc and its device-wide synchronisation is
not acceptable). Its scratch is one fixed device array shared by all calls.

The test calls the entry point through the C ABI twice in a row, on two
different read sets, and checks each result bit-exact (integer output, so the
tolerance is zero) against the allocating entry point on the same input. The
second call must not see anything the first one left in the shared array.
It also checks the documented edges: inputs above the maximum numbers of
reads and of k-mer occurrences are refused, output arrays too small return
the survivor count needed, a call with no reads returns an empty graph, and
a small call followed by a larger one (a larger table region) leaves nothing
behind. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import swapgb
from common import kat_text, synth_case_text

pytestmark = pytest.mark.gpu


def _fn():
    f = swapgb.lib().swg_build_device_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(swapgb.Opts), C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                  C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    return f


def _device_reads(text: bytes, k: int):
    import torch
    r = swapgb.reads_from_fasta(text, k)
    p = torch.from_numpy(r.packed.view(np.int32).copy()).cuda()
    o = torch.from_numpy(r.off.view(np.int64).copy()).cuda()
    ln = torch.from_numpy(r.len.view(np.int32).copy()).cuda()
    return r, p, o, ln


def _call(text: bytes, k: int, c: int, cap: int | None = None):
    import torch
    r, p, o, ln = _device_reads(text, k)
    if cap is None:
        cap = max(1, int((r.len.astype(np.int64) - k + 1).clip(min=0).sum()))
    keys = torch.zeros(max(cap, 1), dtype=torch.int64, device="cuda")
    mult = torch.zeros(max(cap, 1), dtype=torch.int64, device="cuda")
    n = C.c_uint64()
    torch.cuda.synchronize()
    st = _fn()(C.byref(swapgb.Opts(k=k, cutoff=c)), p.data_ptr(), p.numel(), o.data_ptr(),
               ln.data_ptr(), o.numel(), keys.data_ptr(), mult.data_ptr(), cap, C.byref(n))
    return st, n.value, keys, mult


def _noalloc_records(text: bytes, k: int, c: int):
    st, n, keys, mult = _call(text, k, c)
    assert st == 0, swapgb.lib().swg_last_error().decode()
    n = C.c_uint64(n)
    kk = keys[: n.value].cpu().numpy().view(np.uint64)
    mm = mult[: n.value].cpu().numpy().view(np.uint8).reshape(-1, 8)
    order = np.argsort(kk, kind="stable")
    return kk[order], mm[order]


def _allocating_records(text: bytes, k: int, c: int):
    g = swapgb.Graph()
    g.build_reads(swapgb.Opts(k=k, cutoff=c), swapgb.reads_from_fasta(text, k))
    return g.copy_out(sorted=True)


def test_noalloc_matches_allocating_build_twice_in_a_row():
    cases = [(synth_case_text("c2_small"), 31, 5), (kat_text("orient_k19"), 19, 1)]
    for text, k, c in cases:
        got_k, got_m = _noalloc_records(text, k, c)
        want_k, want_m = _allocating_records(text, k, c)
        assert got_k.size == want_k.size
        assert np.array_equal(got_k, want_k)
        assert np.array_equal(got_m, want_m)


def test_noalloc_rejects_inputs_above_its_maximum():
    n = C.c_uint64()
    st = _fn()(C.byref(swapgb.Opts(k=31, cutoff=5)), 1, 1, 1, 1, (1 << 20) + 1, 0, 0, 0, C.byref(n))
    assert st == 1
    assert b"at most" in swapgb.lib().swg_last_error()


def test_noalloc_small_call_then_larger_call():
    # the second call's table region is larger than the first's: entries the
    # first call left past its own region must not leak into the second
    cases = [(kat_text("tandem_k21"), 21, 2), (kat_text("orient_k19"), 19, 0),
             (synth_case_text("c2_small"), 31, 5)]
    for text, k, c in cases:
        got_k, got_m = _noalloc_records(text, k, c)
        want_k, want_m = _allocating_records(text, k, c)
        assert np.array_equal(got_k, want_k) and np.array_equal(got_m, want_m)


def test_noalloc_output_too_small_reports_the_count_needed():
    text, k, c = synth_case_text("c2_small"), 31, 5
    want_k, _ = _allocating_records(text, k, c)
    assert want_k.size > 1
    st, n, _, _ = _call(text, k, c, cap=1)
    assert st == 1 and n == want_k.size
    assert b"too small" in swapgb.lib().swg_last_error()


def test_noalloc_no_reads():
    n = C.c_uint64(7)
    st = _fn()(C.byref(swapgb.Opts(k=31, cutoff=5)), 0, 0, 0, 0, 0, 0, 0, 0, C.byref(n))
    assert st == 0 and n.value == 0


def test_noalloc_rejects_occurrences_above_its_maximum():
    # two reads of 1,258,283 bases at k = 31: 2,516,506 occurrences, one past
    # the 2,516,505 the fixed table holds at 60% load
    rng = np.random.default_rng(5)
    seq = lambda: bytes(np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, 1_258_283)])
    text = b">a\n" + seq() + b"\n>b\n" + seq() + b"\n"
    st, n, _, _ = _call(text, 31, 5, cap=16)
    assert st == 1 and n == 0
    assert b"occurrences" in swapgb.lib().swg_last_error()
    # and one occurrence fewer is built
    st, n, _, _ = _call(text[:-2] + b"\n", 31, 5, cap=1 << 22)
    assert st == 0, swapgb.lib().swg_last_error().decode()
