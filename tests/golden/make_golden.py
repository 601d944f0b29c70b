"""Generate the golden fixtures in this folder from KFR 7.0.1 itself.

Run in a checkout where the reference sources exist (they are compiled into oracle/_ref/libkfr_ref.so by
`make -C oracle ref`):

    python tests/golden/make_golden.py

Every fixture stores the seeded input and the reference's output for it, so the tests can pin both the
C restatement (oracle/) and the GPU library against the reference without the reference present.
Inputs are numpy PCG64 streams generated in float64 (not KFR's own PRNG, whose stream depends on the SIMD
width).  Outputs come from KFR's dft_plan<double>/<float>, dft_plan_real, dct_plan, convolve, correlate and
convolve_filter.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle.oracle import Oracle, build  # noqa: E402

SEED = 20261203

# complex sizes: every N in 1..64 (radix 2..10 stages, generic primes), KFR's special 48/60, Bluestein
# primes (>= 101) and the mixed-radix lengths of the parity configs.
COMPLEX_SIZES = list(range(1, 65)) + [
    72, 96, 100, 101, 121, 127, 128, 210, 243, 256, 343, 625, 1000, 1024, 1536, 2187, 4096, 8191, 9990,
]
REAL_SIZES = [2, 4, 6, 8, 10, 16, 30, 64, 100, 254, 256, 1920, 4096]
# DCT sizes where the reference's dct_plan is correct (power-of-two and single-stage plans).  For
# mixed-radix lengths with more than two stages (100, 1000, ...) KFR's dft_execute places its scratch at
# temp + temp_size (src/dft/fft-impl.hpp:1962-1964), which dct_plan has enlarged by its own 2N buffer
# (include/kfr/dft/fft.hpp:929), so the DFT scratch overwrites the mirrored input and the output is not a
# DCT; those sizes are pinned against the documented formula instead.
DCT_SIZES = [1, 2, 3, 4, 5, 7, 8, 16, 17, 32, 127, 509, 512, 1024]


def main() -> None:
    build(ref=True)
    ref = Oracle("ref")
    rng = np.random.default_rng(SEED)

    # ---- complex DFT, f64 and f32 --------------------------------------------------------------
    fx = {}
    for n in COMPLEX_SIZES:
        batch = 2 if n < 4096 else 1
        x = rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))
        fx[f"x_{n}"] = x
        fx[f"fwd64_{n}"] = ref.dft(x, False)
        fx[f"inv64_{n}"] = ref.dft(x, True)
        x32 = x.astype(np.complex64)
        fx[f"fwd32_{n}"] = ref.dft(x32, False, precision="f32")
        fx[f"inv32_{n}"] = ref.dft(x32, True, precision="f32")
    np.savez_compressed(os.path.join(HERE, "dft_complex.npz"), sizes=np.array(COMPLEX_SIZES), **fx)

    # ---- real DFT (CCs and Perm), forward and inverse ---------------------------------------------
    fr = {}
    for n in REAL_SIZES:
        x = rng.standard_normal((2, n))
        fr[f"x_{n}"] = x
        for fmt, ccs in (("ccs", True), ("perm", False)):
            X = ref.dft_real(x, ccs)
            fr[f"fwd_{fmt}_{n}"] = X
            # inverse of a general (non-Hermitian DC/Nyquist) spectrum: only the real parts of those bins
            # are used by the reference
            S = rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape)
            fr[f"spec_{fmt}_{n}"] = S
            fr[f"inv_{fmt}_{n}"] = ref.dft_real_inverse(S, n, ccs)
    np.savez_compressed(os.path.join(HERE, "dft_real.npz"), sizes=np.array(REAL_SIZES), **fr)

    # ---- DCT-II / DCT-III -------------------------------------------------------------------------
    fd = {}
    for n in DCT_SIZES:
        x = rng.uniform(-1, 1, (2, n))
        fd[f"x_{n}"] = x
        fd[f"fwd_{n}"] = ref.dct(x, False)
        fd[f"inv_{n}"] = ref.dct(x, True)
    np.savez_compressed(os.path.join(HERE, "dct.npz"), sizes=np.array(DCT_SIZES), **fd)

    # ---- convolve / correlate ----------------------------------------------------------------------
    fc = {}
    pairs = [(5, 5), (1, 1), (100, 7), (1000, 1023), (3, 300), (4096, 33)]
    for i, (na, nb) in enumerate(pairs):
        a = rng.standard_normal(na)
        b = rng.standard_normal(nb)
        ac = a + 1j * rng.standard_normal(na)
        bc = b + 1j * rng.standard_normal(nb)
        fc[f"a_{i}"], fc[f"b_{i}"], fc[f"ac_{i}"], fc[f"bc_{i}"] = a, b, ac, bc
        for corr in (0, 1):
            fc[f"real_{corr}_{i}"] = ref.convolve(a, b, bool(corr))
            fc[f"cplx_{corr}_{i}"] = ref.convolve(ac, bc, bool(corr))
    fc["npairs"] = np.array(len(pairs))

    # ---- convolve_filter: streaming with uneven chunks, state carried across calls, then reset ------
    cases = [
        (5, 1024, [5]),
        (1023, 1024, [4096, 1000, 3, 2048]),
        (3000, 256, [1000, 7, 777, 5000]),
        (1, 16, [5, 100]),
        (700, 64, [64, 1, 300, 1023]),
    ]
    for i, (nt, blk, chunks) in enumerate(cases):
        for kind in ("real", "cplx"):
            t = rng.standard_normal(nt)
            if kind == "cplx":
                t = t + 1j * rng.standard_normal(nt)
            f = ref.filter(t, blk)
            fc[f"ftaps_{kind}_{i}"] = t
            fc[f"fblock_{kind}_{i}"] = np.array(blk)
            for j, c in enumerate(chunks):
                x = rng.standard_normal(c)
                if kind == "cplx":
                    x = x + 1j * rng.standard_normal(c)
                fc[f"fin_{kind}_{i}_{j}"] = x
                fc[f"fout_{kind}_{i}_{j}"] = f.process(x)
            f.reset()
            x = rng.standard_normal(300)
            if kind == "cplx":
                x = x + 1j * rng.standard_normal(300)
            fc[f"fin_{kind}_{i}_reset"] = x
            fc[f"fout_{kind}_{i}_reset"] = f.process(x)
            fc[f"fnchunks_{kind}_{i}"] = np.array(len(chunks))
    fc["nfilters"] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, "convolution.npz"), **fc)

    # ---- multi-dimensional complex and real DFT (dft_plan_md / dft_plan_md_real) ---------------------
    fm = {}
    md_shapes = [(4, 8), (3, 5, 7), (16, 16), (6, 10), (2, 3, 4, 5), (1, 7), (8, 1), (32, 6), (5, 2, 2, 3, 2)]
    for i, shp in enumerate(md_shapes):
        x = rng.uniform(-1, 1, shp) + 1j * rng.uniform(-1, 1, shp)
        fm[f"x_{i}"] = x
        fm[f"fwd_{i}"] = ref.dft_md(x)
        fm[f"inv_{i}"] = ref.dft_md(x, inverse=True)
    fm["n"] = np.array(len(md_shapes))
    md_real_shapes = [(4, 8), (3, 5, 6), (16, 16), (6, 10), (2, 3, 4, 6), (7, 2), (1, 12)]
    for i, shp in enumerate(md_real_shapes):
        x = rng.standard_normal(shp)
        fm[f"rx_{i}"] = x
        X = ref.dft_md_real(x)
        fm[f"rfwd_{i}"] = X
        S = rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape)
        fm[f"rspec_{i}"] = S
        fm[f"rinv_{i}"] = ref.dft_md_real(S, inverse=True, shape=shp)
    fm["nr"] = np.array(len(md_real_shapes))
    np.savez_compressed(os.path.join(HERE, "dft_md.npz"), **fm)
    fft_multiply_fixture(ref)
    fir_fixture(ref)
    print("golden fixtures written to", HERE)


FIR_TAPS = [1, 5, 31, 256, 1023, 4097]


def fir_fixture(ref) -> None:
    """fir_filter<double> (include/kfr/dsp/fir.hpp, src/dsp/fir.cpp:54-57) streaming over uneven chunks,
    then reset, from its own seeded stream."""
    rng = np.random.default_rng(SEED + 6)
    ff = {"ntaps": np.array(FIR_TAPS)}
    chunks = [1, 700, 3001, 64, 5000]
    for m in FIR_TAPS:
        taps = rng.standard_normal(m) / np.sqrt(m)
        xs = [rng.standard_normal(c) for c in chunks]
        xr = rng.standard_normal(2000)
        ff[f"taps_{m}"] = taps
        for j, x in enumerate(xs):
            ff[f"in_{m}_{j}"] = x
        ff[f"in_{m}_reset"] = xr
        f = ref.fir(taps)
        for j, x in enumerate(xs):
            ff[f"out_{m}_{j}"] = f.process(x)
        f.reset()
        ff[f"out_{m}_reset"] = f.process(xr)
    ff["nchunks"] = np.array(len(chunks))
    np.savez_compressed(os.path.join(HERE, "fir.npz"), **ff)


def fft_multiply_fixture(ref) -> None:
    """fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020), CCs and Perm, f32 and f64,
    from their own seeded stream so that the other fixtures do not change when this one is added."""
    rng = np.random.default_rng(SEED + 5)
    ff = {}
    n = 1025  # a 2048-point real spectrum in CCs; Perm uses the first 1024 elements
    for prec, dt in (("f64", np.complex128), ("f32", np.complex64)):
        a, b, c = ((rng.uniform(-1, 1, (3, n)) + 1j * rng.uniform(-1, 1, (3, n))).astype(dt) for _ in range(3))
        ff[f"a_{prec}"], ff[f"b_{prec}"], ff[f"c_{prec}"] = a, b, c
        for fmt, m in (("ccs", n), ("perm", n - 1)):
            perm = fmt == "perm"
            ff[f"mul_{fmt}_{prec}"] = ref.fft_multiply(a[:, :m], b[:, :m], perm=perm)
            ff[f"mac_{fmt}_{prec}"] = ref.fft_multiply(a[:, :m], b[:, :m], acc=c[:, :m], perm=perm)
    np.savez_compressed(os.path.join(HERE, "fft_multiply.npz"), **ff)


if __name__ == "__main__":
    if sys.argv[1:] == ["fft_multiply"]:
        build(ref=True)
        fft_multiply_fixture(Oracle("ref"))
    elif sys.argv[1:] == ["fir"]:
        build(ref=True)
        fir_fixture(Oracle("ref"))
    else:
        main()
