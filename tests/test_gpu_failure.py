"""Failure detection without a GPU fault: every wait of a kernel is bounded, and a wait that runs out
turns into an error message on the host, after which the same plan works again.

Each persistent pipelined kernel waits on an mbarrier for the bulk copy of its next tile; the uneven
batch's tiles wait on stage counters.  kfr_set_wait_limit(0) makes every such wait give up at its first
poll (the copy itself still lands: the kernel drains it before its CTA exits), and the uneven-batch test
hook makes every dependent tile wait for one more tile than its stage has, a count nothing reaches.  The
error reaches kfr_last_error() through the plan's device flag, the convention of the reference's C API
(src/capi/capi.cpp:36-91)."""
import time

import numpy as np
import pytest

from oracle.oracle import c32_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu

DEFAULT = 1 << 22


@pytest.fixture
def restore_limit():
    yield
    k.lib().kfr_set_wait_limit(DEFAULT)


@pytest.mark.parametrize("n,batch", [(4096, 600), (8192, 300), (8191, 300), (65536, 40), (127, 5000)])
def test_copy_wait_that_runs_out_is_reported_and_plan_recovers(restore_limit, orc, n, batch):
    """k_c2c_pipe (4096), k_c2c_reg (8192), k_rader_pfa (8191, 127) and the tensor-copy four-step passes
    (65536 = 256 x 256)."""
    plan = k.dft_plan(n)
    g = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    y = torch.zeros_like(x)
    tmp = torch.empty(max(1, plan.temp_size_batch(batch)), dtype=torch.uint8, device="cuda")
    L = k.lib()
    assert L.kfr_set_wait_limit(0) == DEFAULT
    with pytest.raises(k.KfrError, match="gave up waiting"):
        plan.execute_batch(y, x, batch, temp=tmp)
    assert L.kfr_set_wait_limit(DEFAULT) == 0
    plan.execute_batch(y, x, batch, temp=tmp)  # the flag was cleared with the report: this call succeeds
    pick = [0, batch // 2, batch - 1]
    ref = orc.dft(x[pick].cpu().numpy().astype(np.complex128))
    assert rel_rms(y[pick].cpu().numpy(), ref) <= c32_tolerance(n)


@pytest.mark.parametrize("inverse", [False, True])
def test_real_pipelined_wait_reported(restore_limit, orc, inverse):
    """k_r2c_pipe / k_c2r_pipe (N = 1920)."""
    n, batch = 1920, 2000
    plan = k.dft_plan_real(n)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn(batch, n, device="cuda", generator=g)
    X = torch.empty(batch, n // 2 + 1, dtype=torch.complex64, device="cuda")
    plan.execute_batch(X, x, batch)
    L = k.lib()
    L.kfr_set_wait_limit(0)
    with pytest.raises(k.KfrError, match="gave up waiting"):
        if inverse:
            plan.execute_batch(x, X, batch, inverse=True)
        else:
            plan.execute_batch(X, x, batch)
    L.kfr_set_wait_limit(DEFAULT)
    plan.execute_batch(X, x, batch)
    ref = orc.dft_real(x[:4].cpu().numpy().astype(np.float64))
    assert rel_rms(X[:4].cpu().numpy(), ref) <= c32_tolerance(n)


@pytest.mark.parametrize("n", [44100, 48000])
def test_real_fourstep_with_fused_split_wait_reported(restore_limit, orc, n):
    """The real DFT whose split is fused into the four-step row pass (k_fspt_cols over the mirror-paired
    layout, then k_fspt_rows_r2c): a copy wait that runs out is reported, and the plan recovers."""
    batch = 40
    plan = k.dft_plan_real(n)
    g = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn(batch, n, device="cuda", generator=g)
    X = torch.empty(batch, n // 2 + 1, dtype=torch.complex64, device="cuda")
    L = k.lib()
    L.kfr_set_wait_limit(0)
    with pytest.raises(k.KfrError, match="gave up waiting"):
        plan.execute_batch(X, x, batch)
    L.kfr_set_wait_limit(DEFAULT)
    plan.execute_batch(X, x, batch)
    ref = orc.dft_real(x[:3].cpu().numpy().astype(np.float64))
    assert rel_rms(X[:3].cpu().numpy(), ref) <= c32_tolerance(n)


def test_uneven_stage_wait_runs_out_within_a_second(restore_limit, orc):
    """An uneven batch with a four-step signal (65536 = COL tiles, then ROW tiles that wait on the COL
    stage's counter) and one-CTA signals.  With the stage target made unreachable and a limit of 4096 polls
    of 256 ns, the call returns within a second with the error; without the hook the next call is right."""
    lengths = [65536, 1000, 4096, 30720, 127]
    plan = k.dft_plan_uneven(lengths, autotune=False)
    total = sum(lengths)
    g = torch.Generator(device="cuda").manual_seed(9)
    x = torch.randn(total, dtype=torch.complex64, device="cuda", generator=g)
    y = torch.zeros_like(x)
    L = k.lib()
    L.kfr_set_wait_limit(4096)
    L.kfr_dft_uneven_set_unreachable_stage_f32(plan.handle, True)
    t0 = time.perf_counter()
    with pytest.raises(k.KfrError, match="gave up waiting"):
        plan.execute(y, x)
    assert time.perf_counter() - t0 < 1.0
    L.kfr_dft_uneven_set_unreachable_stage_f32(plan.handle, False)
    L.kfr_set_wait_limit(DEFAULT)
    plan.execute(y, x)
    off = 0
    xs, ys = x.cpu().numpy(), y.cpu().numpy()
    for n in lengths:
        ref = orc.dft(xs[off:off + n].astype(np.complex128).reshape(1, n))[0]
        assert rel_rms(ys[off:off + n], ref) <= c32_tolerance(n), n
        off += n


@pytest.mark.parametrize("inverse", [False, True])
def test_dct_pipelined_wait_reported(restore_limit, inverse):
    """k_dct_pipe (DCT-II and DCT-III, N = 512, 4096 signals)."""
    n, batch = 512, 4096
    plan = k.dct_plan(n)
    g = torch.Generator(device="cuda").manual_seed(6)
    x = torch.rand(batch, n, device="cuda", generator=g) * 2 - 1
    y = torch.empty_like(x)
    want = torch.empty_like(x)
    plan.execute_batch(want, x, batch, inverse=inverse)
    L = k.lib()
    L.kfr_set_wait_limit(0)
    with pytest.raises(k.KfrError, match="gave up waiting"):
        plan.execute_batch(y, x, batch, inverse=inverse)
    L.kfr_set_wait_limit(DEFAULT)
    plan.execute_batch(y, x, batch, inverse=inverse)
    assert torch.equal(y, want)
