"""Tensor-core radix-16 plans (split 16-bit operands, FP32 accumulation) beside the FP32 CUDA-core plan on
the precision workload of the tensor-core configuration: N in {2^12, 2^16, 2^20, 2^24} (plus 256), each
signal a seeded sum of 64 sinusoids of random frequency, amplitude and phase plus 1e-3 N(0,1) noise.
Relative RMS error against the FP64 oracle must meet the c32 tolerance 2 log2(N) 2^-24 for both splits and
for the plain plan; max error (relative to the largest output) is reported beside it."""
import numpy as np
import pytest

from oracle.oracle import c32_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def sinusoids(n, batch, seed):
    """Sum of 64 random complex sinusoids plus 1e-3 N(0,1) noise: parameters from a seeded numpy stream, the
    sum evaluated in FP64 on the device (fast at 2^24) and rounded to c32 once."""
    from kfr_gb300.workloads import precision_signals

    return precision_signals(n, batch, seed)


def max_rel(y, ref):
    return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))


SIZES = [(256, 8), (1 << 12, 8), (1 << 16, 4), (1 << 20, 2), (1 << 24, 1)]


@pytest.mark.parametrize("n,batch", SIZES)
def test_tensor_core_and_plain_plans_meet_c32_tolerance(n, batch):
    x = sinusoids(n, batch, n)
    ref = np.fft.fft(x.astype(np.complex128), axis=-1)
    refi = np.fft.ifft(x.astype(np.complex128), axis=-1) * n
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    report = {}
    for name, plan in (("plain", k.dft_plan(n)), ("fp16", k.dft_plan_tensor(n, "fp16")),
                       ("bf16", k.dft_plan_tensor(n, "bf16"))):
        tmp = torch.empty(max(1, plan.temp_size_batch(batch)), dtype=torch.uint8, device="cuda")
        plan.execute_batch(yd, xd, batch, temp=tmp)
        y = yd.cpu().numpy()
        report[name] = (rel_rms(y, ref), max_rel(y, ref))
        plan.execute_batch(yd, xd, batch, temp=tmp, inverse=True)
        report[name + "_inv"] = (rel_rms(yd.cpu().numpy(), refi),)
        if name != "plain":
            assert "tensor-core" in plan.describe()
    for name, errs in report.items():
        assert errs[0] <= c32_tolerance(n), (n, report)


def test_tensor_core_plan_rejects_other_lengths():
    with pytest.raises(k.KfrError, match="256, 4096, 65536"):
        k.dft_plan_tensor(1024)
