"""swg_build_device_noalloc: the build for callers that cannot let the library
allocate device memory (their GPU memory belongs to another allocator or a
fixed budget, or a mid-run cudaMalloc and its device-wide synchronisation is
not acceptable). Its scratch is one fixed device array shared by all calls.

The test calls the entry point through the C ABI twice in a row, on two
different read sets, and checks each result bit-exact (integer output, so the
tolerance is zero) against the allocating entry point on the same input. The
second call must not see anything the first one left in the shared array.
It also checks that inputs above the documented maximum are refused.
This file is collected last on purpose.
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


def _noalloc_records(text: bytes, k: int, c: int):
    import torch
    r, p, o, ln = _device_reads(text, k)
    cap = max(1, int((r.len.astype(np.int64) - k + 1).clip(min=0).sum()))
    keys = torch.zeros(cap, dtype=torch.int64, device="cuda")
    mult = torch.zeros(cap, dtype=torch.int64, device="cuda")
    n = C.c_uint64()
    torch.cuda.synchronize()
    st = _fn()(C.byref(swapgb.Opts(k=k, cutoff=c)), p.data_ptr(), p.numel(), o.data_ptr(),
               ln.data_ptr(), o.numel(), keys.data_ptr(), mult.data_ptr(), cap, C.byref(n))
    assert st == 0, swapgb.lib().swg_last_error().decode()
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
