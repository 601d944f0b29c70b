"""Pins the CPU oracle (oracle/kfr_oracle.c) to KFR 7.0.1 before any GPU result is trusted.

Three sources of truth, none of which needs the reference at run time:
  * the golden fixtures in tests/golden/, produced by KFR itself (tests/golden/make_golden.py);
  * the reference's own known-answer vectors from tests/dft_test.cpp (cited per test);
  * the DFT definition evaluated directly in float64 (numpy), for lengths the fixtures do not cover.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import c32_tolerance, rel_rms

TIGHT = 1e-12  # f64 restatement vs f64 reference


def test_complex_dft_matches_reference_fixtures(orc):
    g = load_golden("dft_complex.npz")
    for n in g["sizes"]:
        x = g[f"x_{n}"]
        assert rel_rms(orc.dft(x), g[f"fwd64_{n}"]) < TIGHT, n
        assert rel_rms(orc.dft(x, inverse=True), g[f"inv64_{n}"]) < TIGHT, n


def test_f32_port_within_c32_tolerance_of_reference(orc):
    """The single-precision port (the CPU baseline) meets the c32 bound against KFR's f64 output, and is
    no worse than 3x KFR's own f32 error on the same input."""
    g = load_golden("dft_complex.npz")
    for n in g["sizes"]:
        x32 = g[f"x_{n}"].astype(np.complex64)
        ref64 = g[f"fwd64_{n}"]
        e_port = rel_rms(orc.dft(x32, precision="f32"), ref64)
        e_kfr = rel_rms(g[f"fwd32_{n}"], ref64)
        assert e_port <= c32_tolerance(n), (n, e_port)
        assert e_port <= max(3 * e_kfr, 1e-7), (n, e_port, e_kfr)


def test_real_dft_matches_reference_fixtures(orc):
    g = load_golden("dft_real.npz")
    for n in g["sizes"]:
        n = int(n)
        x = g[f"x_{n}"]
        for fmt, ccs in (("ccs", True), ("perm", False)):
            assert rel_rms(orc.dft_real(x, ccs), g[f"fwd_{fmt}_{n}"]) < TIGHT, (n, fmt)
            got = orc.dft_real_inverse(g[f"spec_{fmt}_{n}"], n, ccs)
            assert rel_rms(got, g[f"inv_{fmt}_{n}"]) < TIGHT, (n, fmt)


def test_dct_matches_reference_fixtures(orc):
    g = load_golden("dct.npz")
    for n in g["sizes"]:
        x = g[f"x_{n}"]
        assert rel_rms(orc.dct(x), g[f"fwd_{n}"]) < TIGHT, n
        assert rel_rms(orc.dct(x, inverse=True), g[f"inv_{n}"]) < TIGHT, n


def _dct2_direct(x):
    n = x.shape[-1]
    k = np.arange(n)[:, None]
    m = np.arange(n)[None, :]
    return x @ np.cos(np.pi * k * (2 * m + 1) / (2 * n)).T


def _dct3_direct(x):
    n = x.shape[-1]
    m = np.arange(n)[:, None]
    k = np.arange(n)[None, :]
    w = np.ones(n)
    w[0] = 0.5
    return (x * w) @ np.cos(np.pi * k * (2 * m + 1) / (2 * n)).T


@pytest.mark.parametrize("n", [6, 10, 100, 600, 1000, 1200])
def test_dct_mixed_radix_follows_documented_formula(orc, n):
    """At mixed-radix lengths the reference's dct_plan output is corrupted by its own DFT scratch (see
    tests/golden/make_golden.py); the oracle follows the formula dct_plan documents instead
    (include/kfr/dft/fft.hpp:926: unscaled DCT-II; inverse = DCT-III with X0/2)."""
    x = np.random.default_rng(n).uniform(-1, 1, (2, n))
    assert rel_rms(orc.dct(x), _dct2_direct(x)) < 1e-12
    assert rel_rms(orc.dct(x, inverse=True), _dct3_direct(x)) < 1e-12


def test_dct_known_answer_16():
    """tests/dft_test.cpp:396-423: dct_plan<float>(16) on 0..15, tolerance 1e-5 (rms)."""
    from oracle.oracle import Oracle

    orc = Oracle("orc")
    x = np.arange(16, dtype=np.float32)
    fwd = np.array([120.0, -51.79283109806667, 0.0, -5.6781471211595695, 0.0, -1.9843883778092053, 0.0,
                    -0.9603691873838152, 0.0, -0.5308329190495176, 0.0, -0.3030379000702155, 0.0,
                    -0.1584982220313824, 0.0, -0.0494839805703826])
    inv = np.array([59.00747544192212, -65.54341437693878, 27.70332758523579, -24.56124678824279,
                    15.546989102481612, -14.293082621965974, 10.08224348063459, -9.38097406470581,
                    6.795411054455922, -6.320715753372687, 4.455202292297903, -4.0896421269390455,
                    2.580439536964837, -2.2695816108369176, 0.9311870090070382, -0.643618159997807])
    for prec in ("f32", "f64"):
        assert np.sqrt(np.mean((orc.dct(x, precision=prec) - fwd) ** 2)) < 1e-5
        assert np.sqrt(np.mean((orc.dct(x, inverse=True, precision=prec) - inv) ** 2)) < 1e-5


def test_convolve_known_answers(orc):
    """tests/dft_test.cpp:107-165: convolve / correlate of 5-point vectors, rms < 1e-4."""
    a = np.array([1, 2, 3, 4, 5], dtype=np.float64)
    b = np.array([0.25, 0.5, 1.0, -2.0, 1.5])
    conv = np.array([0.25, 1.0, 2.75, 2.5, 3.75, 3.5, 1.5, -4.0, 7.5])
    corr = np.array([1.5, 1.0, 1.5, 2.5, 3.75, -4.0, 7.75, 3.5, 1.25])
    assert np.sqrt(np.mean((orc.convolve(a, b) - conv) ** 2)) < 1e-4
    assert np.sqrt(np.mean((orc.convolve(a, b, correlate=True) - corr) ** 2)) < 1e-4
    ca, cb = a.astype(np.complex128), b.astype(np.complex128)
    assert np.sqrt(np.mean(np.abs(orc.convolve(ca, cb) - conv) ** 2)) < 1e-4
    assert np.sqrt(np.mean(np.abs(orc.convolve(ca, cb, correlate=True) - corr) ** 2)) < 1e-4


def test_convolve_filter_known_answers(orc):
    """tests/dft_test.cpp:127-152: convolve_filter on 5 samples; state carries over; reset() clears it."""
    a = np.array([1, 2, 3, 4, 5], dtype=np.float64)
    b = np.array([0.25, 0.5, 1.0, -2.0, 1.5])
    want = np.array([0.25, 1.0, 2.75, 2.5, 3.75])
    f = orc.filter(a)
    assert np.sqrt(np.mean((f.process(b) - want) ** 2)) < 1e-4
    fc = orc.filter(a.astype(np.complex128))
    assert np.sqrt(np.mean(np.abs(fc.process(b.astype(np.complex128)) - want) ** 2)) < 1e-4
    assert np.sqrt(np.mean(np.abs(fc.process(b.astype(np.complex128)) - want) ** 2)) > 1e-4
    fc.reset()
    assert np.sqrt(np.mean(np.abs(fc.process(b.astype(np.complex128)) - want) ** 2)) < 1e-4


def test_convolve_matches_reference_fixtures(orc):
    g = load_golden("convolution.npz")
    for i in range(int(g["npairs"])):
        for corr in (0, 1):
            got = orc.convolve(g[f"a_{i}"], g[f"b_{i}"], correlate=bool(corr))
            assert rel_rms(got, g[f"real_{corr}_{i}"]) < TIGHT
            got = orc.convolve(g[f"ac_{i}"], g[f"bc_{i}"], correlate=bool(corr))
            assert rel_rms(got, g[f"cplx_{corr}_{i}"]) < TIGHT


def test_convolve_filter_streaming_matches_reference_fixtures(orc):
    g = load_golden("convolution.npz")
    for i in range(int(g["nfilters"])):
        for kind in ("real", "cplx"):
            f = orc.filter(g[f"ftaps_{kind}_{i}"], int(g[f"fblock_{kind}_{i}"]))
            for j in range(int(g[f"fnchunks_{kind}_{i}"])):
                got = f.process(g[f"fin_{kind}_{i}_{j}"])
                assert rel_rms(got, g[f"fout_{kind}_{i}_{j}"]) < 1e-11, (i, kind, j)
            f.reset()
            got = f.process(g[f"fin_{kind}_{i}_reset"])
            assert rel_rms(got, g[f"fout_{kind}_{i}_reset"]) < 1e-11, (i, kind)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 11, 13, 97, 101, 211, 1009, 9988, 9999, 96001, 1 << 16])
def test_complex_dft_against_definition(orc, n):
    """Lengths outside the fixtures, including fft_reconstruction's 9988..9999 and 96001 ranges
    (tests/dft_test.cpp:181-221), against numpy's float64 FFT."""
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (1, n)) + 1j * rng.uniform(-1, 1, (1, n))
    assert rel_rms(orc.dft(x), np.fft.fft(x)) < 1e-13
    assert rel_rms(orc.dft(x, inverse=True), np.fft.ifft(x) * n) < 1e-13


def test_reconstruction(orc):
    """tests/dft_test.cpp:181-221: forward then inverse / N reproduces a sinusoid (rms < 1e-6, max < 1e-5)."""
    for n in list(range(2, 40)) + [9988, 9999, 96001]:
        x = np.sin(np.arange(n) * 0.1) + 0j
        y = orc.dft(orc.dft(x.astype(np.complex64), precision="f32"), inverse=True, precision="f32") / n
        d = np.abs(y - x)
        assert np.sqrt(np.mean(d ** 2)) < 1e-6 and d.max() < 1e-5, n


def test_real_dft_requires_even_size(orc):
    """include/kfr/dft/fft.hpp:485: dft_plan_real requires size to be even."""
    with pytest.raises(ValueError):
        orc.dft_real(np.zeros(7))


def test_fft_multiply_matches_reference_fixtures(orc):
    """fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020), both packings, against
    the reference's own outputs: products agree to the last bits (one rounding of a complex product)."""
    f = load_golden("fft_multiply.npz")
    for prec, eps in (("f64", 2.0**-52), ("f32", 2.0**-23)):
        a, b, c = f[f"a_{prec}"], f[f"b_{prec}"], f[f"c_{prec}"]
        for fmt, m in (("ccs", a.shape[1]), ("perm", a.shape[1] - 1)):
            perm = fmt == "perm"
            got = orc.fft_multiply(a[:, :m], b[:, :m], perm=perm)
            assert np.max(np.abs(got - f[f"mul_{fmt}_{prec}"])) <= 4 * eps
            got = orc.fft_multiply(a[:, :m], b[:, :m], acc=c[:, :m], perm=perm)
            assert np.max(np.abs(got - f[f"mac_{fmt}_{prec}"])) <= 8 * eps
            # Perm: element 0 is the part-by-part product (DC and Nyquist are both real)
            if perm:
                want0 = a[:, 0].real * b[:, 0].real + 1j * a[:, 0].imag * b[:, 0].imag
                assert np.allclose(f[f"mul_{fmt}_{prec}"][:, 0], want0, rtol=4 * eps)


def test_fir_matches_reference_fixtures(orc):
    """The direct-form FIR restatement against KFR's own fir_filter<double> (src/dsp/fir.cpp:54-57):
    streaming over uneven chunks with the delay line kept across calls, then reset."""
    g = load_golden("fir.npz")
    for m in g["ntaps"]:
        f = orc.fir(g[f"taps_{m}"])
        for j in range(int(g["nchunks"])):
            assert rel_rms(f.process(g[f"in_{m}_{j}"]), g[f"out_{m}_{j}"]) <= TIGHT, (m, j)
        f.reset()
        assert rel_rms(f.process(g[f"in_{m}_reset"]), g[f"out_{m}_reset"]) <= TIGHT, m
