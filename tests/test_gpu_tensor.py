"""Tensor-core radix-16 plans (split hi + lo BF16 / FP16 operands, FP32 accumulation) beside the FP32
CUDA-core plan, on the precision workload: each signal a seeded sum of 64 sinusoids of random frequency,
amplitude and phase plus 1e-3 N(0,1) noise.  Relative RMS and max error against the FP64 oracle."""
import numpy as np
import pytest

from oracle.oracle import c32_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def sinusoids(n, batch, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(n)
    x = np.zeros((batch, n), np.complex128)
    for b in range(batch):
        f = rng.uniform(0, n, 64)
        a = rng.uniform(0, 1, 64)
        ph = rng.uniform(0, 2 * np.pi, 64)
        x[b] = (a[:, None] * np.exp(1j * (2 * np.pi * f[:, None] * t[None, :] / n + ph[:, None]))).sum(0)
    x += 1e-3 * (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n)))
    return x.astype(np.complex64)


def max_rel(y, ref):
    return float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))


# bounds on relative RMS (measured: FP16 hi + lo 5e-7 at 256 and 1.5e-6 at 4096, BF16 hi + lo 4-5e-6, the
# FP32 CUDA-core plan 1e-7): FP16 keeps 22 significant bits but its low parts of small values go subnormal
BOUNDS = {"fp16": 3e-6, "bf16": 2e-5}


@pytest.mark.parametrize("n", [256, 4096])
@pytest.mark.parametrize("split", ["fp16", "bf16"])
def test_tensor_core_plan_accuracy(orc, n, split):
    batch = 64
    x = sinusoids(n, batch, n)
    ref = orc.dft(x.astype(np.complex128), threads=8)
    refi = orc.dft(x.astype(np.complex128), inverse=True, threads=8)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    plain = k.dft_plan(n)
    plain.execute_batch(yd, xd, batch)
    e_plain = rel_rms(yd.cpu().numpy(), ref)
    assert e_plain <= c32_tolerance(n)
    tc = k.dft_plan_tensor(n, split)
    assert "tensor-core" in tc.describe()
    tc.execute_batch(yd, xd, batch)
    y = yd.cpu().numpy()
    e_tc, m_tc = rel_rms(y, ref), max_rel(y, ref)
    assert e_tc <= BOUNDS[split], (split, e_tc, m_tc, e_plain)
    tc.execute_batch(yd, xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy(), refi) <= BOUNDS[split]


def test_tensor_core_plan_rejects_other_lengths():
    with pytest.raises(k.KfrError, match="256 and 4096"):
        k.dft_plan_tensor(1024)
