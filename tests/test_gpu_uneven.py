"""Uneven batch: many signals of different lengths back to back in one persistent launch (graph-replayed),
against the oracle and against the plain form (one plan execution per signal)."""
import numpy as np
import pytest

from oracle.oracle import c32_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402
from kfr_gb300.workloads import uneven_lengths  # noqa: E402

pytestmark = pytest.mark.gpu


def _signals(lengths, seed):
    rng = np.random.default_rng(seed)
    total = int(sum(lengths))
    x = (rng.uniform(-1, 1, total) + 1j * rng.uniform(-1, 1, total)).astype(np.complex64)
    return x


def _check_against_oracle(orc, lengths, x, y, inverse, pick):
    offs = np.concatenate([[0], np.cumsum(lengths)])
    for i in pick:
        n = lengths[i]
        ref = orc.dft(x[offs[i]:offs[i] + n].astype(np.complex128).reshape(1, n), inverse=inverse)[0]
        assert rel_rms(y[offs[i]:offs[i] + n], ref) <= c32_tolerance(max(n, 2)), (i, n)


@pytest.mark.parametrize("autotune", [False, True])
def test_uneven_small_against_oracle(orc, autotune):
    lengths = uneven_lengths(300, seed=7) + [1, 2, 3, 17, 4096, 8192, 8191, 12000, 65536, 65537]
    x = _signals(lengths, 1)
    plan = k.dft_plan_uneven(lengths, autotune=autotune)
    assert plan.size == sum(lengths)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    for inverse in (False, True):
        plan.execute(yd, xd, inverse=inverse)
        _check_against_oracle(orc, lengths, x, yd.cpu().numpy(), inverse, range(len(lengths)))


def test_uneven_full_batch_matches_plain_form_and_replays(orc):
    """8192 signals, log-uniform lengths on [64, 65536] (7-smooth, 10% prime): the persistent launch agrees
    with one plain execution per signal; the captured graph replays identically; new pointers re-capture."""
    lengths = uneven_lengths(8192)
    x = _signals(lengths, 2)
    plan = k.dft_plan_uneven(lengths, autotune=True)
    d = plan.describe()
    assert "8192 signals" in d
    xd = torch.from_numpy(x).cuda()
    y1 = torch.empty_like(xd)
    y2 = torch.empty_like(xd)
    plan.execute(y1, xd)
    plan.execute(y2, xd)  # graph replay
    assert torch.equal(y1, y2)
    yp = torch.empty_like(xd)
    plan.execute_per_signal(yp, xd)
    nmax = max(lengths)
    assert rel_rms(y1.cpu().numpy(), yp.cpu().numpy().astype(np.complex128)) <= c32_tolerance(nmax)
    # different output buffer: captured again
    y3 = torch.zeros_like(xd)
    plan.execute(y3, xd)
    assert torch.equal(y1, y3)
    rng = np.random.default_rng(3)
    _check_against_oracle(orc, lengths, x, y1.cpu().numpy(), False, rng.choice(len(lengths), 40, replace=False))


def test_uneven_rejects_host_pointers():
    plan = k.dft_plan_uneven([8, 12])
    x = np.zeros(20, np.complex64)
    with pytest.raises(k.KfrError, match="device pointers"):
        plan.execute(x, x)
