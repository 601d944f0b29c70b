"""Adjoint kernels behind the C ABI, wrapped in torch.autograd.Function (here only, in the test harness).

Each gradient is checked three ways:
  * torch.autograd.gradcheck on double-precision plans: central finite differences of the GPU forward
    against the GPU adjoint;
  * single-precision adjoints against gradients assembled from the oracle's CPU transforms (the reference's
    algorithms in double precision) at the differentiable-ops shapes: DCT-II of 4096 x 512, a real-DFT
    magnitude loss at N = 4096 x 2048, FIR filtering of 2^20-sample signals with 1023 taps;
  * directional derivatives against double-precision central finite differences of the oracle's forward.
Complex gradients follow complex autograd: dL/dRe(z) + i dL/dIm(z).
"""
import numpy as np
import pytest

from oracle.oracle import c32_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def _sfx(t):
    return "f64" if t.dtype in (torch.float64, torch.complex128) else "f32"


class DFT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, plan, inverse):
        x = x.contiguous()
        y = torch.empty_like(x)
        plan.execute_batch(y, x, x.shape[0], inverse=inverse)
        ctx.plan, ctx.inverse = plan, inverse
        return y

    @staticmethod
    def backward(ctx, gy):
        gx = torch.empty_like(gy)
        ctx.plan.adjoint_batch(gx, gy.contiguous(), gy.shape[0], inverse=ctx.inverse)
        return gx, None, None


class RealDFT(torch.autograd.Function):
    """Forward real DFT (x real, batch x N) -> CCs / Perm spectrum."""

    @staticmethod
    def forward(ctx, x, plan, bins):
        x = x.contiguous()
        cdt = torch.complex128 if x.dtype == torch.float64 else torch.complex64
        y = torch.empty((x.shape[0], bins), dtype=cdt, device=x.device)
        plan.execute_batch(y, x, x.shape[0])
        ctx.plan, ctx.n = plan, x.shape[1]
        return y

    @staticmethod
    def backward(ctx, gy):
        rdt = torch.float64 if gy.dtype == torch.complex128 else torch.float32
        gx = torch.empty((gy.shape[0], ctx.n), dtype=rdt, device=gy.device)
        ctx.plan.adjoint_batch(gx, gy.contiguous(), gy.shape[0])
        return gx, None, None


class RealIDFT(torch.autograd.Function):
    """Inverse real DFT (spectrum -> batch x N reals)."""

    @staticmethod
    def forward(ctx, Y, plan, n):
        Y = Y.contiguous()
        rdt = torch.float64 if Y.dtype == torch.complex128 else torch.float32
        x = torch.empty((Y.shape[0], n), dtype=rdt, device=Y.device)
        plan.execute_batch(x, Y, Y.shape[0], inverse=True)
        ctx.plan, ctx.bins = plan, Y.shape[1]
        return x

    @staticmethod
    def backward(ctx, gx):
        cdt = torch.complex128 if gx.dtype == torch.float64 else torch.complex64
        gY = torch.empty((gx.shape[0], ctx.bins), dtype=cdt, device=gx.device)
        ctx.plan.adjoint_batch(gY, gx.contiguous(), gx.shape[0], inverse=True)
        return gY, None, None


class DCT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, plan, inverse):
        x = x.contiguous()
        y = torch.empty_like(x)
        plan.execute_batch(y, x, x.shape[0], inverse=inverse)
        ctx.plan, ctx.inverse = plan, inverse
        return y

    @staticmethod
    def backward(ctx, gy):
        gx = torch.empty_like(gy)
        ctx.plan.adjoint_batch(gx, gy.contiguous(), gy.shape[0], inverse=ctx.inverse)
        return gx, None, None


class FIR(torch.autograd.Function):
    """Causal FIR filtering of each row of x (channels x n) by a convolution filter from a reset state."""

    @staticmethod
    def forward(ctx, x, taps, block):
        x, taps = x.contiguous(), taps.contiguous()
        y = torch.empty_like(x)
        f = k.convolve_filter(taps, block, dtype=_sfx(x))
        for c in range(x.shape[0]):
            f.reset()
            f.apply(y[c], x[c])
        ctx.save_for_backward(x, taps)
        return y

    @staticmethod
    def backward(ctx, gy):
        x, taps = ctx.saved_tensors
        gx = torch.empty_like(x)
        gh = torch.empty_like(taps)
        k.fir_backward(taps, x, gy.contiguous(), gx, gh, channels=x.shape[0])
        return gx, gh, None


# ------------------------------------------------------------------------------------------------------
# finite differences of the GPU forward (double precision) against the GPU adjoint
# ------------------------------------------------------------------------------------------------------

def _gc(fn, *inputs):
    # the full Jacobian for small inputs; random projections (gradcheck's fast mode) for larger ones
    fast = sum(t.numel() for t in inputs) > 256
    assert torch.autograd.gradcheck(fn, inputs, eps=1e-6, atol=1e-6, rtol=1e-5, nondet_tol=1e-12, fast_mode=fast)


@pytest.mark.parametrize("n", [12, 16, 127, 1000])
@pytest.mark.parametrize("inverse", [False, True])
def test_gradcheck_complex_dft(n, inverse):
    plan = k.dft_plan(n, "f64")
    x = torch.randn(3, n, dtype=torch.complex128, device="cuda", requires_grad=True)
    _gc(lambda t: DFT.apply(t, plan, inverse), x)


@pytest.mark.parametrize("n", [16, 20, 1920])
@pytest.mark.parametrize("fmt", ["CCs", "Perm"])
def test_gradcheck_real_dft(n, fmt):
    plan = k.dft_plan_real(n, fmt, "f64")
    bins = n // 2 + 1 if fmt == "CCs" else n // 2
    x = torch.randn(2, n, dtype=torch.float64, device="cuda", requires_grad=True)
    _gc(lambda t: RealDFT.apply(t, plan, bins), x)
    Y = torch.randn(2, bins, dtype=torch.complex128, device="cuda", requires_grad=True)
    _gc(lambda t: RealIDFT.apply(t, plan, n), Y)


@pytest.mark.parametrize("n", [10, 16, 512])
@pytest.mark.parametrize("inverse", [False, True])
def test_gradcheck_dct(n, inverse):
    plan = k.dct_plan(n, "f64")
    x = torch.randn(3, n, dtype=torch.float64, device="cuda", requires_grad=True)
    _gc(lambda t: DCT.apply(t, plan, inverse), x)


def test_gradcheck_fir():
    x = torch.randn(2, 40, dtype=torch.float64, device="cuda", requires_grad=True)
    h = torch.randn(7, dtype=torch.float64, device="cuda", requires_grad=True)
    _gc(lambda a, b: FIR.apply(a, b, 8), x, h)


# ------------------------------------------------------------------------------------------------------
# single precision against gradients built from the oracle's CPU transforms, at the differentiable-ops shapes
# ------------------------------------------------------------------------------------------------------

def test_dct2_gradient_4096x512_against_oracle(orc):
    rng = np.random.default_rng(51)
    x = rng.uniform(-1, 1, (4096, 512)).astype(np.float32)
    w = rng.uniform(-1, 1, (4096, 512)).astype(np.float32)
    plan = k.dct_plan(512)
    xt = torch.from_numpy(x).cuda().requires_grad_()
    loss = (DCT.apply(xt, plan, False) * torch.from_numpy(w).cuda()).sum()
    loss.backward()
    # d/dx sum(w * C x) = C^T w = DCT-III of w with the first term at full weight
    w2 = w.astype(np.float64)
    w2[:, 0] *= 2
    ref = orc.dct(w2, inverse=True, threads=8)
    assert rel_rms(xt.grad.cpu().numpy(), ref) <= 2 * c32_tolerance(512)


def test_real_dft_magnitude_loss_gradient_4096x2048_against_oracle(orc):
    rng = np.random.default_rng(52)
    n, batch = 4096, 2048
    x = rng.standard_normal((batch, n)).astype(np.float32)
    plan = k.dft_plan_real(n)
    xt = torch.from_numpy(x).cuda().requires_grad_()
    Y = RealDFT.apply(xt, plan, n // 2 + 1)
    Y.abs().sum().backward()
    # gradient of sum|Y_k| w.r.t. Y is Y/|Y|; back through the real DFT: c2r with bins 1..N/2-1 halved
    Yd = orc.dft_real(x.astype(np.float64), threads=8)
    g = Yd / np.abs(Yd)
    g[:, 1:-1] *= 0.5
    ref = orc.dft_real_inverse(g, n, threads=8)
    assert rel_rms(xt.grad.cpu().numpy(), ref) <= 4 * c32_tolerance(n)


def _kaiser_lowpass(m, cutoff, beta):
    t = np.arange(m) - (m - 1) / 2
    h = 2 * cutoff * np.sinc(2 * cutoff * t) * np.kaiser(m, beta)
    return h / h.sum()


def test_fir_gradients_1023_taps_against_oracle(orc):
    """FFT convolution of 2^20-sample signals with a 1023-tap Kaiser lowpass (+1e-2 noise), loss = sum y^2:
    gradients with respect to signal and taps on 4 signals (the 64-signal case is timed, not re-derived
    on the CPU)."""
    rng = np.random.default_rng(53)
    chans, n, m = 4, 1 << 20, 1023
    x = rng.standard_normal((chans, n)).astype(np.float32)
    h = (_kaiser_lowpass(m, 0.2, 3.0) + 1e-2 * rng.standard_normal(m)).astype(np.float32)
    xt = torch.from_numpy(x).cuda().requires_grad_()
    ht = torch.from_numpy(h).cuda().requires_grad_()
    y = FIR.apply(xt, ht, 1024)
    (y * y).sum().backward()
    # reference: y = causal FIR; g = 2y; grad_x[t] = sum_m h[m] g[t+m]; grad_h[m] = sum_c sum_t g[t] x[t-m]
    x64, h64 = x.astype(np.float64), h.astype(np.float64)
    gx_ref = np.empty_like(x64)
    gh_ref = np.zeros(m)
    for c in range(chans):
        yc = orc.convolve(x64[c], h64)[:n]
        g = 2 * yc
        gx_ref[c] = orc.convolve(g, h64, correlate=True)[m - 1:m - 1 + n]
        gh_ref += orc.convolve(g, x64[c], correlate=True)[n - 1:n - 1 + m]
    assert rel_rms(xt.grad.cpu().numpy(), gx_ref) <= 8 * c32_tolerance(n)
    assert rel_rms(ht.grad.cpu().numpy(), gh_ref) <= 8 * c32_tolerance(n)


# ------------------------------------------------------------------------------------------------------
# directional derivatives against double-precision central differences of the oracle's forward
# ------------------------------------------------------------------------------------------------------

def test_complex_dft_directional_derivative_fp64(orc):
    rng = np.random.default_rng(54)
    n, batch = 1536, 16
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    w = rng.uniform(0.5, 1.5, (batch, n))
    plan = k.dft_plan(n)
    xt = torch.from_numpy(x).cuda().requires_grad_()
    y = DFT.apply(xt, plan, False)
    (torch.from_numpy(w).cuda().float() * y.abs() ** 2).sum().backward()
    g = xt.grad.cpu().numpy().astype(np.complex128)

    def loss(z):
        return float(np.sum(w * np.abs(orc.dft(z, threads=8)) ** 2))

    for seed in range(3):
        v = np.random.default_rng(100 + seed).standard_normal((batch, n, 2)) @ np.array([1, 1j])
        eps = 1e-4
        x64 = x.astype(np.complex128)
        fd = (loss(x64 + eps * v) - loss(x64 - eps * v)) / (2 * eps)
        an = float(np.sum(g.real * v.real + g.imag * v.imag))
        assert abs(fd - an) <= 1e-4 * abs(fd), (fd, an)
