"""FIR filter plans (kfr_filter_create_fir_plan_*, the reference's fir_filter<T>: src/capi/capi.cpp:567-580)
through the C ABI, computed by the FFT convolution path, against KFR's own direct-form fir_filter<double>
outputs (tests/golden/fir.npz): streaming over uneven chunks with the state kept across calls, then reset.

Error bound: each output block is a forward real FFT of F points, one product with the taps' spectrum and
an inverse real FFT, with F = next_pow2(4 (M - 1)) but at least 2048 (twice the 1024-sample block).  Its
relative RMS error is that of three F-point transforms, 3 x the per-transform tolerance (c32: 2 log2(F)
2^-24; c64: 4 log2(F) 2^-53); by Parseval the relative error of the spectrum is the relative error of y."""
import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import c32_tolerance, c64_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def fft_points(m):
    f = 2048
    while f < 4 * (m - 1):
        f *= 2
    return f


def bound(m, sfx):
    return 3 * (c32_tolerance if sfx == "f32" else c64_tolerance)(fft_points(m))


@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_fir_streaming_matches_reference(sfx):
    g = load_golden("fir.npz")
    rdt = np.float32 if sfx == "f32" else np.float64
    for m in g["ntaps"]:
        f = k.fir_filter(g[f"taps_{m}"].astype(rdt))
        for j in range(int(g["nchunks"])):
            x = g[f"in_{m}_{j}"].astype(rdt)
            y = np.zeros_like(x)
            f.apply(y, x)
            assert rel_rms(y, g[f"out_{m}_{j}"]) <= bound(m, sfx), (m, j, rel_rms(y, g[f"out_{m}_{j}"]))
        f.reset()
        x = g[f"in_{m}_reset"].astype(rdt)
        y = np.zeros_like(x)
        f.apply(y, x)
        assert rel_rms(y, g[f"out_{m}_reset"]) <= bound(m, sfx), m


def test_fir_device_buffers_long_signal(orc):
    """A 511-tap FIR over 2^20 device samples in three calls, against the oracle's direct form in FP64."""
    rng = np.random.default_rng(21)
    m, n = 511, 1 << 20
    taps = (rng.standard_normal(m) / np.sqrt(m)).astype(np.float32)
    x = rng.standard_normal(n).astype(np.float32)
    want = orc.fir(taps.astype(np.float64)).process(x.astype(np.float64))
    f = k.fir_filter(taps)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    cuts = [0, 1000, 600000, n]
    for a, b in zip(cuts[:-1], cuts[1:]):
        f.apply(yd[a:b], xd[a:b])
    assert rel_rms(yd.cpu().numpy(), want) <= bound(m, "f32")
