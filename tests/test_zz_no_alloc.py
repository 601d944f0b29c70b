"""kfr_dft_execute_static_scratch_f32: the allocation-free entry point.

Callers that must not allocate GPU memory while they run (real-time threads, code under CUDA stream
capture, hosts that reserve all device memory up front) use this entry point instead of
kfr_dft_execute_batch_f32, which allocates plan-owned scratch on first use.  Its scratch is one fixed
device array of KFR_STATIC_SCRATCH_BYTES (32 MiB).  This test calls it through the C ABI on a two-pass
(four-step) length that needs scratch, twice in a row, and checks each result against the regular entry
point within the c32 tolerance used by every parity test; it also checks that the calls allocate no device
memory and that oversized requests and host pointers are rejected with a message.

The file name sorts last so that a run stopping at its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from oracle.oracle import c32_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu

STATIC_SCRATCH_BYTES = 32 << 20


def _static(plan, batch, out, inp, inverse=False, stream=None):
    L = k.lib()
    L.kfr_dft_execute_static_scratch_f32(plan.handle, batch, out.data_ptr(), inp.data_ptr(), inverse, stream)
    return L.kfr_last_error()


def test_static_scratch_matches_regular_entry_point_twice():
    n, batch = 1 << 18, 4  # four-step: 8 MiB of scratch
    plan = k.dft_plan(n, "f32")
    assert plan.temp_size_batch(batch) == batch * n * 8 <= STATIC_SCRATCH_BYTES
    g = torch.Generator(device="cuda").manual_seed(42)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    want = torch.empty_like(x)
    plan.execute_batch(want, x, batch)
    for inverse in (False, True):
        if inverse:
            plan.execute_batch(want, x, batch, inverse=True)
        for call in range(2):
            got = torch.full_like(x, float("nan"))
            assert _static(plan, batch, got, x, inverse) == b""
            err = rel_rms(got.cpu().numpy(), want.cpu().numpy().astype(np.complex128))
            assert err <= c32_tolerance(n), (inverse, call, err)


def test_static_scratch_allocates_nothing():
    n, batch = 1 << 20, 3  # 24 MiB of scratch
    plan = k.dft_plan(n, "f32")
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    assert _static(plan, batch, y, x) == b""  # first call on this device: one-time set-up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _static(plan, batch, y, x) == b""
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_before - free_after < (1 << 20), (free_before, free_after)
    # and on a stream
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        assert _static(plan, batch, y, x, stream=s.cuda_stream) == b""
    s.synchronize()
    want = torch.empty_like(x)
    plan.execute_batch(want, x, batch)
    assert rel_rms(y.cpu().numpy(), want.cpu().numpy().astype(np.complex128)) <= c32_tolerance(n)


def test_static_scratch_rejects_oversize_and_host_pointers():
    n = 1 << 20
    plan = k.dft_plan(n, "f32")
    batch = STATIC_SCRATCH_BYTES // (n * 8) + 1
    x = torch.zeros(batch, n, dtype=torch.complex64, device="cuda")
    err = _static(plan, batch, x, x)
    assert b"static scratch" in err
    hx = np.zeros(n, dtype=np.complex64)
    L = k.lib()
    L.kfr_dft_execute_static_scratch_f32(plan.handle, 1, hx.ctypes.data, hx.ctypes.data, False, None)
    assert b"device pointers" in L.kfr_last_error()


def test_static_scratch_single_pass_plan_needs_no_scratch():
    n, batch = 4096, 8
    plan = k.dft_plan(n, "f32")
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda")
    y, want = torch.empty_like(x), torch.empty_like(x)
    assert _static(plan, batch, y, x) == b""
    plan.execute_batch(want, x, batch)
    assert rel_rms(y.cpu().numpy(), want.cpu().numpy().astype(np.complex128)) <= c32_tolerance(n)
