"""GPU parity of the DFT path, called through the C ABI (libkfr_capi.so via the kfr_gb300 ctypes mirror).

Checked against:
  * the golden fixtures produced by KFR 7.0.1 itself (tests/golden/), at every length they hold;
  * the CPU oracle (oracle/, pinned to the same fixtures) at lengths and batches the fixtures do not hold.
Tolerances bound the relative RMS error against a double-precision reference:
  c32: 2 * log2(N) * 2^-24        c64: 4 * log2(N) * 2^-53   (N >= 2)
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import c32_tolerance, c64_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def tol(n, sfx):
    return c32_tolerance(n) if sfx == "f32" else c64_tolerance(n)


def cdt(sfx):
    return np.complex64 if sfx == "f32" else np.complex128


def tdt(sfx):
    return torch.complex64 if sfx == "f32" else torch.complex128


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


# ------------------------------------------------------------------------------------------------------
# Complex DFT
# ------------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_complex_dft_reference_fixtures_host_buffers(sfx):
    """Single-signal kfr_dft_execute / kfr_dft_execute_inverse with host (numpy) buffers at every fixture
    length: all radix 2..16 codelets, generic primes 17..61, Bluestein (101, 127, 8191), KFR's 48/60."""
    g = load_golden("dft_complex.npz")
    for n in g["sizes"]:
        n = int(n)
        plan = k.dft_plan(n, sfx)
        assert plan.size == n
        for b in range(g[f"x_{n}"].shape[0]):
            x = g[f"x_{n}"][b].astype(cdt(sfx))
            out = np.zeros_like(x)
            plan.execute(out, x)
            assert rel_rms(out, g[f"fwd64_{n}"][b]) <= tol(n, sfx), (n, rel_rms(out, g[f"fwd64_{n}"][b]))
            plan.execute(out, x, inverse=True)
            assert rel_rms(out, g[f"inv64_{n}"][b]) <= tol(n, sfx), n


@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_complex_dft_reference_fixtures_device_batched(sfx):
    g = load_golden("dft_complex.npz")
    for n in g["sizes"]:
        n = int(n)
        x = g[f"x_{n}"].astype(cdt(sfx))
        xd = dev(x)
        yd = torch.empty_like(xd)
        plan = k.dft_plan(n, sfx)
        plan.execute_batch(yd, xd, x.shape[0])
        assert rel_rms(yd.cpu().numpy(), g[f"fwd64_{n}"]) <= tol(n, sfx), n
        plan.execute_batch(yd, xd, x.shape[0], inverse=True)
        assert rel_rms(yd.cpu().numpy(), g[f"inv64_{n}"]) <= tol(n, sfx), n


# lengths x batch: the mixed-radix / prime parity set, multi-signal CTAs, four-step and multi-kernel Bluestein
BATCHED = [(4096, 64), (1000, 37), (1536, 21), (2187, 15), (30720, 3), (127, 70), (8191, 4), (16384, 3),
           (65536, 2), (9990, 5), (17 * 19 * 23, 3), (2 * 3 * 5 * 7 * 11 * 13, 2), (1 << 20, 1),
           (40009, 2), (3 * 65537, 1), (1, 5), (2, 9), (3, 7)]


@pytest.mark.parametrize("n,batch", BATCHED)
@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_complex_dft_batched_against_oracle(orc, n, batch, sfx):
    rng = np.random.default_rng(n * 7 + batch)
    x = (rng.uniform(-1, 1, (batch, n)) + 1j * rng.uniform(-1, 1, (batch, n))).astype(cdt(sfx))
    ref = orc.dft(x.astype(np.complex128), threads=8)
    refi = orc.dft(x.astype(np.complex128), inverse=True, threads=8)
    plan = k.dft_plan(n, sfx)
    xd = dev(x)
    yd = torch.empty_like(xd)
    plan.execute_batch(yd, xd, batch)
    assert rel_rms(yd.cpu().numpy(), ref) <= tol(n, sfx), (n, rel_rms(yd.cpu().numpy(), ref))
    plan.execute_batch(yd, xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy(), refi) <= tol(n, sfx), n
    # in place
    zd = xd.clone()
    plan.execute_batch(zd, zd, batch)
    assert rel_rms(zd.cpu().numpy(), ref) <= tol(n, sfx), n


@pytest.mark.parametrize("n,batch", [(127, 40000), (8191, 500), (127, 40001), (8191, 301), (8191, 1), (127, 1)])
def test_rader_tiles_many_per_cta(orc, n, batch):
    """Prime lengths through the persistent Rader kernel with several tiles per CTA (tile buffers
    reused, output bulk stores overlapping the next tile's load), a shorter last tile, a batch whose end is
    8 bytes past a 16-byte boundary (the last element loaded separately), forward, inverse, in place, and
    from an 8-byte-misaligned pointer (which takes the plain kernel)."""
    rng = np.random.default_rng(n + batch)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    pick = np.unique(np.r_[0:3, batch // 2, batch - 3:batch].clip(0, batch - 1))
    ref = orc.dft(x[pick].astype(np.complex128), threads=8)
    refi = orc.dft(x[pick].astype(np.complex128), inverse=True, threads=8)
    plan = k.dft_plan(n, "f32")
    d = plan.describe()
    assert "prime-factor" in d, d  # the persistent kernel over tiles of signals
    xd = dev(x)
    yd = torch.empty_like(xd)
    plan.execute_batch(yd, xd, batch)
    assert rel_rms(yd.cpu().numpy()[pick], ref) <= tol(n, "f32")
    full = yd.clone()
    plan.execute_batch(yd, xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy()[pick], refi) <= tol(n, "f32")
    zd = xd.clone()
    plan.execute_batch(zd, zd, batch)
    assert torch.equal(zd, full)
    # misaligned by one element: same results through the plain kernel
    buf = torch.empty(batch * n + 1, dtype=torch.complex64, device="cuda")
    buf[1:].copy_(xd.reshape(-1))
    out = torch.empty_like(buf)
    plan.execute_batch(out[1:], buf[1:], batch)
    got = out[1:].reshape(batch, n).cpu().numpy()
    assert rel_rms(got, full.cpu().numpy()) <= tol(n, "f32")


@pytest.mark.parametrize("n,batch", [(16384, 400), (8192, 500), (16384, 1)])
def test_one_signal_per_cta_persistent(orc, n, batch):
    """Lengths that run one signal per persistent CTA with the signal in registers (the next signal's bulk
    copy lands while the last pass stores): several signals per CTA, forward, inverse, in place, and from an
    8-byte-misaligned pointer (which takes the per-signal kernel)."""
    rng = np.random.default_rng(n + batch)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    pick = np.unique(np.r_[0:2, batch // 2, batch - 2:batch].clip(0, batch - 1))
    ref = orc.dft(x[pick].astype(np.complex128), threads=8)
    refi = orc.dft(x[pick].astype(np.complex128), inverse=True, threads=8)
    plan = k.dft_plan(n, "f32")
    assert "persistent one per CTA" in plan.describe()
    xd = dev(x)
    yd = torch.empty_like(xd)
    plan.execute_batch(yd, xd, batch)
    assert rel_rms(yd.cpu().numpy()[pick], ref) <= tol(n, "f32")
    full = yd.clone()
    plan.execute_batch(yd, xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy()[pick], refi) <= tol(n, "f32")
    zd = xd.clone()
    plan.execute_batch(zd, zd, batch)
    assert torch.equal(zd, full)
    buf = torch.empty(batch * n + 1, dtype=torch.complex64, device="cuda")
    buf[1:].copy_(xd.reshape(-1))
    out = torch.empty_like(buf)
    plan.execute_batch(out[1:], buf[1:], batch)
    got = out[1:].reshape(batch, n).cpu().numpy()
    assert rel_rms(got, full.cpu().numpy()) <= tol(n, "f32")


@pytest.mark.parametrize("n,batch", [(30720, 300), (24000, 200), (65536, 150), (1 << 18, 40), (1 << 20, 12),
                                     (22050, 200), (1 << 22, 3), (1 << 24, 1)])
def test_fourstep_pair_tiles_many_per_cta(orc, n, batch):
    """Four-step lengths whose column and row passes run as persistent kernels fed by 2-D tensor copies
    (160 x 192, 150 x 160, 256 x 256 in two passes; 512 x 512, 1024 x 1024, 2048 x 2048 and 4096 x 4096 on
    16-, 8-, 4- and 2-wide tiles in three passes, boxes of 256 rows; the 147-point column pass of 147 x 150):
    several tiles per CTA, ragged row
    tiles (150 rows in tiles of 16), forward, inverse, in place, and from an 8-byte-misaligned pointer (which
    takes the per-tile kernels)."""
    rng = np.random.default_rng(n + batch)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    pick = np.unique(np.r_[0:2, batch // 2, batch - 2:batch].clip(0, batch - 1))
    ref = orc.dft(x[pick].astype(np.complex128), threads=8)
    refi = orc.dft(x[pick].astype(np.complex128), inverse=True, threads=8)
    plan = k.dft_plan(n, "f32")
    assert "compile-time pair" in plan.describe()
    xd = dev(x)
    yd = torch.empty_like(xd)
    plan.execute_batch(yd, xd, batch)
    assert rel_rms(yd.cpu().numpy()[pick], ref) <= tol(n, "f32")
    full = yd.clone()
    plan.execute_batch(yd, xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy()[pick], refi) <= tol(n, "f32")
    zd = xd.clone()
    plan.execute_batch(zd, zd, batch)
    assert torch.equal(zd, full)
    buf = torch.empty(batch * n + 1, dtype=torch.complex64, device="cuda")
    buf[1:].copy_(xd.reshape(-1))
    out = torch.empty_like(buf)
    plan.execute_batch(out[1:], buf[1:], batch)
    got = out[1:].reshape(batch, n).cpu().numpy()
    assert rel_rms(got, full.cpu().numpy()) <= tol(n, "f32")


@pytest.mark.parametrize("n,batch", [(1000, 3000), (4096, 700), (127, 9000), (2187, 400), (1021, 300), (1536, 1),
                                     (8191, 300), (30720, 70), (16384, 90)])
def test_page_locked_host_buffers(orc, n, batch):
    """Page-locked host input and output (torch pin_memory): one-CTA lengths up to 4096 points (pipelined,
    Rader, Bluestein) are read and written by the kernels across the host link with plain loads and stores
    (zero-copy), longer ones go through the chunk pipeline; forward and inverse against the device call's
    results, the oracle on a few signals, and in place."""
    rng = np.random.default_rng(n + batch)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    plan = k.dft_plan(n, "f32")
    xd = dev(x)
    hx = torch.from_numpy(x).pin_memory()
    for inverse in (False, True):
        yd = torch.empty_like(xd)
        plan.execute_batch(yd, xd, batch, inverse=inverse)
        hy = torch.empty_like(hx).pin_memory()
        plan.execute_batch(hy, hx, batch, inverse=inverse)
        assert rel_rms(hy.numpy(), yd.cpu().numpy()) <= tol(n, "f32") / 4, inverse
    pick = np.unique(np.r_[0, batch // 2, batch - 1])
    ref = orc.dft(x[pick].astype(np.complex128), threads=8)
    assert rel_rms(plan_forward(plan, hx, batch)[pick], ref) <= tol(n, "f32")
    hz = hx.clone().pin_memory()
    plan.execute_batch(hz, hz, batch)
    assert rel_rms(hz.numpy()[pick], ref) <= tol(n, "f32")


@pytest.mark.parametrize("n,batch", [(1000, 600), (8191, 40)])
def test_kfr_allocate_buffers(orc, n, batch):
    """Buffers from kfr_allocate (host memory registered with the driver): a zero-copy length (1000) and a
    chunk-pipeline length (8191) give the device call's results."""
    import ctypes
    nbytes = batch * n * 8
    pin, pout = k.allocate(nbytes), k.allocate(nbytes)
    try:
        hin = np.ctypeslib.as_array((ctypes.c_float * (2 * batch * n)).from_address(pin)).view(np.complex64)
        hout = np.ctypeslib.as_array((ctypes.c_float * (2 * batch * n)).from_address(pout)).view(np.complex64)
        rng = np.random.default_rng(n)
        hin[:] = (rng.standard_normal(batch * n) + 1j * rng.standard_normal(batch * n)).astype(np.complex64)
        plan = k.dft_plan(n, "f32")
        plan.execute_batch(pout, pin, batch)
        xd = dev(hin.reshape(batch, n))
        yd = torch.empty_like(xd)
        plan.execute_batch(yd, xd, batch)
        assert rel_rms(hout.reshape(batch, n), yd.cpu().numpy()) <= tol(n, "f32") / 4
        pick = [0, batch - 1]
        ref = orc.dft(hin.reshape(batch, n)[pick].astype(np.complex128))
        assert rel_rms(hout.reshape(batch, n)[pick], ref) <= tol(n, "f32")
    finally:
        k.deallocate(pin)
        k.deallocate(pout)


def plan_forward(plan, hx, batch):
    hy = torch.empty_like(hx).pin_memory()
    plan.execute_batch(hy, hx, batch)
    return hy.numpy()


@pytest.mark.parametrize("n,batch", [(1000, 5000), (8191, 700), (4096, 1100)])
def test_host_buffers_pipelined_match_device(n, batch):
    """Host input and output (the reference's calling convention) split into chunks that overlap copies with
    transforms: same results as the device-resident call, forward and inverse, for complex, real and DCT
    plans."""
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    plan = k.dft_plan(n, "f32")
    for inverse in (False, True):
        y = np.empty_like(x)
        plan.execute_batch(y, x, batch, inverse=inverse)
        xd = dev(x)
        yd = torch.empty_like(xd)
        plan.execute_batch(yd, xd, batch, inverse=inverse)
        assert rel_rms(y, yd.cpu().numpy()) <= tol(n, "f32") / 4, inverse
    if n % 2 == 0:
        r = rng.standard_normal((batch, n)).astype(np.float32)
        rp = k.dft_plan_real(n)
        c = np.empty((batch, n // 2 + 1), np.complex64)
        rp.execute_batch(c, r, batch)
        cd = torch.empty((batch, n // 2 + 1), dtype=torch.complex64, device="cuda")
        rp.execute_batch(cd, dev(r), batch)
        assert rel_rms(c, cd.cpu().numpy()) <= tol(n, "f32") / 4
        back = np.empty_like(r)
        rp.execute_batch(back, c, batch, inverse=True)
        assert rel_rms(back / n, r) <= 2 * tol(n, "f32")
        dp = k.dct_plan(n)
        d = np.empty_like(r)
        dp.execute_batch(d, r, batch)
        dd = torch.empty_like(dev(r))
        dp.execute_batch(dd, dev(r), batch)
        assert rel_rms(d, dd.cpu().numpy()) <= tol(n, "f32") / 4


@pytest.mark.parametrize("n", [1 << 24, 30720000])
def test_complex_dft_large_single(orc, n):
    """The large single transforms of the mixed-radix parity set (c32)."""
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    ref = orc.dft(x.astype(np.complex128).reshape(1, n))[0]
    plan = k.dft_plan(n, "f32")
    xd = dev(x)
    yd = torch.empty_like(xd)
    plan.execute(yd, xd)
    assert rel_rms(yd.cpu().numpy(), ref) <= c32_tolerance(n)
    # round trip through the inverse: x * N
    plan.execute(yd, yd, inverse=True)
    assert rel_rms(yd.cpu().numpy() / n, x) <= 2 * c32_tolerance(n)


def test_complex_dft_c64_large(orc):
    n = 1 << 20
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = orc.dft(x.reshape(1, n))[0]
    plan = k.dft_plan(n, "f64")
    xd = dev(x)
    yd = torch.empty_like(xd)
    plan.execute(yd, xd)
    assert rel_rms(yd.cpu().numpy(), ref) <= c64_tolerance(n)


@pytest.mark.parametrize("n", [1000, 1536, 2187, 30720, 127, 8191])
def test_complex_dft_linearity_and_parseval_full_batch(orc, n):
    """Size-independent properties at the benchmark's full batch of each mixed-radix length (256 MiB of
    c32): linearity, Parseval per signal, the inverse of the forward (x N) over the whole batch, and the
    oracle on the first and last signals."""
    batch = (256 << 20) // (8 * n)
    g = torch.Generator(device="cuda").manual_seed(5)
    a = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    b = torch.randn(batch, n, dtype=torch.complex64, device="cuda", generator=g)
    plan = k.dft_plan(n, "f32")
    fa, fb, fab = torch.empty_like(a), torch.empty_like(b), torch.empty_like(a)
    plan.execute_batch(fa, a, batch)
    plan.execute_batch(fb, b, batch)
    ab = a + 2 * b
    plan.execute_batch(fab, ab, batch)
    err = torch.linalg.vector_norm(fab - (fa + 2 * fb)) / torch.linalg.vector_norm(fab)
    assert err.item() <= 4 * c32_tolerance(n)
    # Parseval: sum |X|^2 = N sum |x|^2 (per signal)
    ea = (a.abs() ** 2).double().sum(dim=1) * n
    eA = (fa.abs() ** 2).double().sum(dim=1)
    assert torch.max(torch.abs(eA / ea - 1)).item() < 1e-5
    # the inverse of the forward gives x N back for every signal of the batch
    back = torch.empty_like(a)
    plan.execute_batch(back, fa, batch, inverse=True)
    err = torch.linalg.vector_norm(back / n - a) / torch.linalg.vector_norm(a)
    assert err.item() <= 2 * c32_tolerance(n)
    pick = [0, batch - 1]
    ref = orc.dft(a[pick].cpu().numpy().astype(np.complex128))
    assert rel_rms(fa[pick].cpu().numpy(), ref) <= c32_tolerance(n)


@pytest.mark.parametrize("n", [1920, 44100, 48000])
def test_real_dft_round_trip_and_parseval_full_batch(orc, n):
    """The real lengths of the mixed-radix set at the benchmark's full batch (256 MiB of f32): Parseval per
    signal (|X_0|^2 + 2 sum |X_k|^2 + |X_N/2|^2 = N sum x^2), the inverse of the forward (x N) over the whole
    batch, and the oracle on the first and last signals."""
    batch = (256 << 20) // (4 * n)
    g = torch.Generator(device="cuda").manual_seed(6)
    x = torch.randn(batch, n, device="cuda", generator=g)
    plan = k.dft_plan_real(n)
    X = torch.empty(batch, n // 2 + 1, dtype=torch.complex64, device="cuda")
    plan.execute_batch(X, x, batch)
    p = (X.abs() ** 2).double()
    eX = p[:, 0] + p[:, -1] + 2 * p[:, 1:-1].sum(dim=1)
    ex = (x.double() ** 2).sum(dim=1) * n
    assert torch.max(torch.abs(eX / ex - 1)).item() < 1e-5
    back = torch.empty_like(x)
    plan.execute_batch(back, X, batch, inverse=True)
    err = torch.linalg.vector_norm(back / n - x) / torch.linalg.vector_norm(x)
    assert err.item() <= 2 * c32_tolerance(n)
    pick = [0, batch - 1]
    ref = orc.dft_real(x[pick].cpu().numpy().astype(np.float64))
    assert rel_rms(X[pick].cpu().numpy(), ref) <= c32_tolerance(n)


def test_plan_queries_and_errors():
    p = k.dft_plan(4096)
    assert p.size == 4096 and p.temp_size == 0
    p2 = k.dft_plan(1 << 20)
    assert p2.temp_size == (1 << 20) * 8  # four-step intermediate
    with pytest.raises(k.KfrError, match="even"):
        k.dft_plan_real(7)
    L = k.lib()
    assert L.kfr_dft_get_size_f32(None) == 0 and b"NULL" in L.kfr_last_error()


def test_caller_provided_device_temp(orc):
    n = 1 << 18
    p = k.dft_plan(n, "f32")
    temp = torch.empty(p.temp_size, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(9)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    out = np.zeros_like(x)
    p.execute(out, x, temp=temp)
    assert rel_rms(out, orc.dft(x.astype(np.complex128).reshape(1, n))[0]) <= c32_tolerance(n)


# ------------------------------------------------------------------------------------------------------
# Real DFT
# ------------------------------------------------------------------------------------------------------

@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_real_dft_reference_fixtures(sfx):
    g = load_golden("dft_real.npz")
    rdt = np.float32 if sfx == "f32" else np.float64
    for n in g["sizes"]:
        n = int(n)
        for fmt in ("ccs", "perm"):
            plan = k.dft_plan_real(n, "CCs" if fmt == "ccs" else "Perm", sfx)
            x = g[f"x_{n}"].astype(rdt)
            X = np.zeros((x.shape[0], plan.complex_size), dtype=cdt(sfx))
            for b in range(x.shape[0]):
                plan.execute(X[b], x[b])
            assert rel_rms(X, g[f"fwd_{fmt}_{n}"]) <= tol(n, sfx), (n, fmt)
            S = g[f"spec_{fmt}_{n}"].astype(cdt(sfx))
            y = np.zeros((S.shape[0], n), dtype=rdt)
            plan.execute_batch(y, S, S.shape[0], inverse=True)
            assert rel_rms(y, g[f"inv_{fmt}_{n}"]) <= tol(n, sfx), (n, fmt)


@pytest.mark.parametrize("n,batch", [(1920, 40), (44100, 3), (48000, 3), (4096, 33), (2048, 17), (2, 5),
                                     (1 << 16, 2), (2 * 8191, 3), (40000, 2), (1920, 5001), (8192, 1201)])
@pytest.mark.parametrize("fmt", ["CCs", "Perm"])
def test_real_dft_batched_against_oracle(orc, n, batch, fmt):
    rng = np.random.default_rng(n + batch)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    ccs = fmt == "CCs"
    ref = orc.dft_real(x.astype(np.float64), ccs=ccs, threads=8)
    plan = k.dft_plan_real(n, fmt, "f32")
    xd = dev(x)
    Xd = torch.empty((batch, plan.complex_size), dtype=torch.complex64, device="cuda")
    plan.execute_batch(Xd, xd, batch)
    assert rel_rms(Xd.cpu().numpy(), ref) <= c32_tolerance(n), n
    yd = torch.empty_like(xd)
    plan.execute_batch(yd, Xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy() / n, x) <= 2 * c32_tolerance(n), n


@pytest.mark.parametrize("n", [44100, 48000])
@pytest.mark.parametrize("fmt", ["CCs", "Perm"])
def test_real_dft_split_fused_into_fourstep_rows(orc, n, fmt):
    """Real lengths whose half-length complex DFT is a compile-time pair (22050 = 147 x 150, 24000 = 150 x 160):
    the column pass writes each column with rows k1 and N1 - k1 side by side (and, for odd N1, one unused slot
    so that the rows stay 16-byte aligned for the row pass's tensor copies), and the row pass applies the
    real split to both rows of each pair, writing the spectrum directly.  Many tiles per CTA, an odd batch,
    both formats; a 4-byte-misaligned input (staged into aligned scratch, then the separate split) gives the
    same results, and so does the inverse into a 4-byte-misaligned output."""
    batch = 61
    rng = np.random.default_rng(n)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    ccs = fmt == "CCs"
    plan = k.dft_plan_real(n, fmt, "f32")
    xd = dev(x)
    Xd = torch.empty((batch, plan.complex_size), dtype=torch.complex64, device="cuda")
    plan.execute_batch(Xd, xd, batch)
    pick = [0, 1, batch // 2, batch - 1]
    ref = orc.dft_real(x[pick].astype(np.float64), ccs=ccs, threads=8)
    assert rel_rms(Xd.cpu().numpy()[pick], ref) <= c32_tolerance(n)
    buf = torch.empty(batch * n + 1, device="cuda")
    buf[1:].copy_(xd.reshape(-1))
    Xm = torch.empty_like(Xd)
    plan.execute_batch(Xm, buf[1:], batch)
    assert rel_rms(Xm.cpu().numpy(), Xd.cpu().numpy()) <= c32_tolerance(n)
    # the inverse into a 4-byte-misaligned output (transformed in place in scratch, then copied)
    back = torch.empty(batch * n + 1, device="cuda")
    plan.execute_batch(back[1:], Xd, batch, inverse=True)
    assert rel_rms(back[1:].reshape(batch, n).cpu().numpy() / n, x) <= 2 * c32_tolerance(n)


@pytest.mark.parametrize("n,batch", [(1920, 33), (4096, 5), (2 * 8191, 3), (30, 7)])
def test_real_dft_reals_aligned_to_one_element(orc, n, batch):
    """Real input and output pointers aligned to one float only (a float array at an odd offset, which the
    reference's float* interface allows): the per-tile kernels load and store such reals one by one, the
    multi-kernel paths stage them through aligned scratch; same results as from aligned buffers."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal((batch, n)).astype(np.float32)
    plan = k.dft_plan_real(n, "CCs", "f32")
    buf = torch.zeros(batch * n + 1, device="cuda")
    buf[1:].copy_(dev(x).reshape(-1))
    X = torch.empty((batch, plan.complex_size), dtype=torch.complex64, device="cuda")
    plan.execute_batch(X, buf[1:], batch)
    ref = orc.dft_real(x.astype(np.float64), ccs=True, threads=8)
    assert rel_rms(X.cpu().numpy(), ref) <= c32_tolerance(n)
    back = torch.zeros(batch * n + 1, device="cuda")
    plan.execute_batch(back[1:], X, batch, inverse=True)
    assert rel_rms(back[1:].reshape(batch, n).cpu().numpy() / n, x) <= 2 * c32_tolerance(n)


# ------------------------------------------------------------------------------------------------------
# DCT
# ------------------------------------------------------------------------------------------------------

def _dct2(x):
    n = x.shape[-1]
    kk = np.arange(n)[:, None]
    m = np.arange(n)[None, :]
    return x @ np.cos(np.pi * kk * (2 * m + 1) / (2 * n)).T


def _dct3(x):
    n = x.shape[-1]
    m = np.arange(n)[:, None]
    kk = np.arange(n)[None, :]
    w = np.ones(n)
    w[0] = 0.5
    return (x * w) @ np.cos(np.pi * kk * (2 * m + 1) / (2 * n)).T


@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_dct_reference_fixtures(sfx):
    g = load_golden("dct.npz")
    rdt = np.float32 if sfx == "f32" else np.float64
    for n in g["sizes"]:
        n = int(n)
        plan = k.dct_plan(n, sfx)
        x = g[f"x_{n}"].astype(rdt)
        y = np.zeros_like(x)
        plan.execute_batch(y, x, x.shape[0])
        assert rel_rms(y, g[f"fwd_{n}"]) <= tol(max(n, 2), sfx), n  # measured at most 0.37 of it
        plan.execute_batch(y, x, x.shape[0], inverse=True)
        assert rel_rms(y, g[f"inv_{n}"]) <= tol(max(n, 2), sfx), n


def test_dct_known_answer_16():
    """tests/dft_test.cpp:396-423 of the reference."""
    plan = k.dct_plan(16)
    x = np.arange(16, dtype=np.float32)
    y = np.zeros(16, dtype=np.float32)
    plan.execute(y, x)
    fwd = np.array([120.0, -51.79283109806667, 0.0, -5.6781471211595695, 0.0, -1.9843883778092053, 0.0,
                    -0.9603691873838152, 0.0, -0.5308329190495176, 0.0, -0.3030379000702155, 0.0,
                    -0.1584982220313824, 0.0, -0.0494839805703826])
    assert np.sqrt(np.mean((y - fwd) ** 2)) < 1e-5


@pytest.mark.parametrize("n,batch", [(512, 4096), (600, 7), (1000, 5), (30720, 2), (127, 9), (1, 3), (3, 4)])
def test_dct_batched_documented_formula(n, batch):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, (batch, n)).astype(np.float32)
    plan = k.dct_plan(n)
    xd = dev(x)
    yd = torch.empty_like(xd)
    x64 = x.astype(np.float64)
    if n <= 4096:
        r2, r3 = _dct2(x64), _dct3(x64)
    else:
        from oracle.oracle import Oracle
        o = Oracle("orc")
        r2, r3 = o.dct(x64), o.dct(x64, inverse=True)
    plan.execute_batch(yd, xd, batch)
    assert rel_rms(yd.cpu().numpy(), r2) <= c32_tolerance(max(n, 2)), n
    plan.execute_batch(yd, xd, batch, inverse=True)
    assert rel_rms(yd.cpu().numpy(), r3) <= c32_tolerance(max(n, 2)), n


# ------------------------------------------------------------------------------------------------------
# FFT convolution filter
# ------------------------------------------------------------------------------------------------------

def test_convolve_filter_known_answer():
    """tests/dft_test.cpp:127-135 of the reference."""
    f = k.convolve_filter(np.array([1, 2, 3, 4, 5], dtype=np.float32))
    x = np.array([0.25, 0.5, 1.0, -2.0, 1.5], dtype=np.float32)
    y = np.zeros(5, dtype=np.float32)
    f.apply(y, x)
    assert np.sqrt(np.mean((y - np.array([0.25, 1.0, 2.75, 2.5, 3.75])) ** 2)) < 1e-4


@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_convolve_filter_streaming_fixtures(sfx):
    """Streaming with uneven chunks, state across calls, then reset() (real filters: the C API's)."""
    g = load_golden("convolution.npz")
    rdt = np.float32 if sfx == "f32" else np.float64
    for i in range(int(g["nfilters"])):
        taps = g[f"ftaps_real_{i}"].astype(rdt)
        f = k.convolve_filter(taps, int(g[f"fblock_real_{i}"]))
        for j in range(int(g[f"fnchunks_real_{i}"])):
            x = g[f"fin_real_{i}_{j}"].astype(rdt)
            y = np.zeros_like(x)
            f.apply(y, x)
            assert rel_rms(y, g[f"fout_real_{i}_{j}"]) <= tol(len(taps) + len(x), sfx), (i, j)
        f.reset()
        x = g[f"fin_real_{i}_reset"].astype(rdt)
        y = np.zeros_like(x)
        f.apply(y, x)
        assert rel_rms(y, g[f"fout_real_{i}_reset"]) <= tol(len(taps) + len(x), sfx), i


def test_convolve_filter_channels_match_single_channel(orc):
    """A 6-channel plan (one launch per call) gives each channel exactly what a one-channel plan gives it,
    across two streaming calls, host and device buffers, and resets every channel's state."""
    rng = np.random.default_rng(12)
    taps = rng.standard_normal(255).astype(np.float32)
    chans, n = 6, 5000
    x = rng.standard_normal((chans, 2 * n)).astype(np.float32)
    multi = k.convolve_filter(taps, 512, channels=chans)
    y = np.empty((chans, n), np.float32)
    outs = []
    for part in (0, 1):
        xp = np.ascontiguousarray(x[:, part * n:(part + 1) * n])
        multi.apply(y, xp)
        outs.append(y.copy())
    got = np.concatenate(outs, axis=1)
    for c in range(chans):
        ref = orc.filter(taps.astype(np.float64), 512).process(x[c].astype(np.float64))
        assert rel_rms(got[c], ref) <= c32_tolerance(2 * n), c
    multi.reset()
    xd = dev(np.ascontiguousarray(x[:, :n]))
    yd = torch.empty_like(xd)
    multi.apply(yd, xd)
    assert np.allclose(yd.cpu().numpy(), outs[0], rtol=0, atol=1e-5)


@pytest.mark.parametrize("sfx,ntaps", [("f32", 20001), ("f64", 10001)])
def test_convolve_filter_taps_longer_than_one_fft(orc, sfx, ntaps):
    """Taps too long for one overlap-save FFT per CTA (the reference's multi-segment case, M >> block):
    whole-call convolutions of [history, input] with the taps, two channels, two streaming calls, reset."""
    rng = np.random.default_rng(ntaps)
    rdt = np.float32 if sfx == "f32" else np.float64
    taps = (rng.standard_normal(ntaps) / np.sqrt(ntaps)).astype(rdt)
    chans, n = 2, 30000
    x = rng.standard_normal((chans, 2 * n)).astype(rdt)
    f = k.convolve_filter(taps, 1024, dtype=sfx, channels=chans)
    outs = []
    for part in (0, 1):
        xd = dev(np.ascontiguousarray(x[:, part * n:(part + 1) * n]))
        yd = torch.empty_like(xd)
        f.apply(yd, xd)
        outs.append(yd.cpu().numpy())
    got = np.concatenate(outs, axis=1)
    tol_f = c32_tolerance if sfx == "f32" else c64_tolerance
    for c in range(chans):
        ref = orc.filter(taps.astype(np.float64), 1024).process(x[c].astype(np.float64))
        assert rel_rms(got[c], ref) <= tol_f(2 * n + ntaps), c
    f.reset()
    xd = dev(np.ascontiguousarray(x[:, :n]))
    yd = torch.empty_like(xd)
    f.apply(yd, xd)
    assert rel_rms(yd.cpu().numpy(), outs[0]) <= tol_f(n + ntaps)


def test_convolve_filter_long_signal_device(orc):
    """1023-tap filter over 2^18 samples in device memory, against the streaming oracle."""
    rng = np.random.default_rng(11)
    taps = rng.standard_normal(1023).astype(np.float32)
    x = rng.standard_normal(1 << 18).astype(np.float32)
    ref = orc.filter(taps.astype(np.float64), 1024).process(x.astype(np.float64))
    f = k.convolve_filter(taps, 1024)
    xd = dev(x)
    yd = torch.empty_like(xd)
    f.apply(yd, xd)
    assert rel_rms(yd.cpu().numpy(), ref) <= c32_tolerance(1 << 18)  # measured 0.09 of it
    # in place on the device
    f.reset()
    zd = xd.clone()
    f.apply(zd, zd)
    assert rel_rms(zd.cpu().numpy(), ref) <= c32_tolerance(1 << 18)
