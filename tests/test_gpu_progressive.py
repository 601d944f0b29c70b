"""Progressive execution (dft_plan<T>::progressive_*, include/kfr/dft/fft.hpp:393-439): one kernel launch
per step.  The number of steps equals the plan's launch count, the result after the last step equals a
one-shot execution of the same plan bit for bit (the same kernels run), host buffers are staged, and the
reference's own test pattern (tests/dft_test.cpp fft_accuracy: start, step until false) gives the DFT."""
import numpy as np
import pytest

from oracle.oracle import c32_tolerance, c64_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 4096, 1000, 127, 8191, 30720, 1 << 16, 1 << 20, 40009, 3 * 65537])
def test_progressive_steps_are_launches_and_match_one_shot(orc, n):
    plan = k.dft_plan(n)
    total = plan.progressive_total_steps()
    assert total == plan.launch_count(1), (total, plan.describe())
    g = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn(n, dtype=torch.complex64, device="cuda", generator=g)
    want = torch.empty_like(x)
    tmp = torch.empty(max(1, plan.temp_size_batch(1)), dtype=torch.uint8, device="cuda")
    x64 = x.cpu().numpy().astype(np.complex128).reshape(1, n)
    for inverse in (False, True):
        plan.execute_batch(want, x, 1, temp=tmp, inverse=inverse)
        got = torch.full_like(x, float("nan"))
        steps = plan.progressive_start(got, x, temp=tmp, inverse=inverse)
        assert steps == total
        done = 0
        while plan.progressive_step(done):
            done += 1
        assert done + 1 == total
        assert torch.equal(got, want), inverse
        ref = orc.dft(x64, inverse=inverse)[0]
        assert rel_rms(got.cpu().numpy(), ref) <= c32_tolerance(n), inverse


@pytest.mark.parametrize("n,sfx", [(30720, "f64"), (1 << 18, "f32"), (4096, "f64")])
def test_progressive_host_buffers(orc, n, sfx):
    """Host input and output, no temp: the input is staged at start, the result copied after the last step."""
    rng = np.random.default_rng(n)
    dt = np.complex64 if sfx == "f32" else np.complex128
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dt)
    y = np.zeros_like(x)
    plan = k.dft_plan(n, sfx)
    steps = plan.progressive_start(y, x)
    assert steps == plan.progressive_total_steps()
    i = 0
    while plan.progressive_step(i):
        assert not np.any(y)  # nothing reaches the host output before the last step
        i += 1
    ref = orc.dft(x.astype(np.complex128).reshape(1, n))[0]
    tol = c32_tolerance(n) if sfx == "f32" else c64_tolerance(n)
    assert rel_rms(y, ref) <= tol


def test_progressive_step_out_of_order_is_an_error():
    plan = k.dft_plan(1024)
    x = torch.zeros(1024, dtype=torch.complex64, device="cuda")
    with pytest.raises(k.KfrError, match="before progressive_start"):
        plan.progressive_step(0)
    plan.progressive_start(x, x)
    with pytest.raises(k.KfrError, match="progressive step 5"):
        plan.progressive_step(5)
