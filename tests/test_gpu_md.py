"""Multi-dimensional DFTs on the GPU through the C ABI (kfr_dft_create_2d/3d/md_plan_*,
kfr_dft_real_create_*_plan_*), against fixtures from KFR's own dft_plan_md / dft_plan_md_real
(tests/golden/dft_md.npz) and against numpy's float64 fftn / rfftn at larger shapes."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import c32_tolerance, c64_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def tol(n, sfx):
    return c32_tolerance(n) if sfx == "f32" else c64_tolerance(n)


@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_md_complex_reference_fixtures(sfx):
    g = load_golden("dft_md.npz")
    cdt = np.complex64 if sfx == "f32" else np.complex128
    for i in range(int(g["n"])):
        x = g[f"x_{i}"].astype(cdt)
        plan = k.dft_plan_md(x.shape, sfx)
        assert plan.size == x.size
        y = np.zeros_like(x)
        plan.execute(y, x)
        assert rel_rms(y, g[f"fwd_{i}"]) <= 2 * tol(x.size, sfx), (x.shape, rel_rms(y, g[f"fwd_{i}"]))
        plan.execute(y, x, inverse=True)
        assert rel_rms(y, g[f"inv_{i}"]) <= 2 * tol(x.size, sfx), x.shape


@pytest.mark.parametrize("sfx", ["f32", "f64"])
def test_md_real_reference_fixtures(sfx):
    g = load_golden("dft_md.npz")
    rdt, cdt = (np.float32, np.complex64) if sfx == "f32" else (np.float64, np.complex128)
    for i in range(int(g["nr"])):
        x = g[f"rx_{i}"].astype(rdt)
        plan = k.dft_plan_md_real(x.shape, dtype=sfx)
        X = np.zeros(plan.complex_shape, dtype=cdt)
        plan.execute(X, x)
        assert rel_rms(X, g[f"rfwd_{i}"]) <= 2 * tol(x.size, sfx), x.shape
        S = g[f"rspec_{i}"].astype(cdt)
        y = np.zeros(x.shape, dtype=rdt)
        plan.execute(y, S, inverse=True)
        assert rel_rms(y, g[f"rinv_{i}"]) <= 2 * tol(x.size, sfx), x.shape


def test_2d_3d_creators_and_large_shapes():
    L = k.lib()
    rng = np.random.default_rng(4)
    for shape in [(1024, 1024), (64, 96, 100), (3, 4096), (2000, 3)]:
        x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
        if len(shape) == 2:
            h = L.kfr_dft_create_2d_plan_f32(*shape)
        else:
            h = L.kfr_dft_create_3d_plan_f32(*shape)
        assert h, L.kfr_last_error()
        xd = torch.from_numpy(x).cuda()
        yd = torch.empty_like(xd)
        L.kfr_dft_execute_f32(h, yd.data_ptr(), xd.data_ptr(), None)
        assert L.kfr_last_error() == b""
        assert rel_rms(yd.cpu().numpy(), np.fft.fftn(x.astype(np.complex128))) <= 2 * c32_tolerance(x.size)
        L.kfr_dft_execute_inverse_f32(h, yd.data_ptr(), yd.data_ptr(), None)
        assert rel_rms(yd.cpu().numpy() / x.size, x) <= 4 * c32_tolerance(x.size)
        L.kfr_dft_delete_plan_f32(h)
    # real 2-D, device buffers, round trip
    shape = (512, 1000)
    x = rng.standard_normal(shape).astype(np.float32)
    plan = k.dft_plan_md_real(shape)
    Xd = torch.empty(plan.complex_shape, dtype=torch.complex64, device="cuda")
    xd = torch.from_numpy(x).cuda()
    plan.execute(Xd, xd)
    assert rel_rms(Xd.cpu().numpy(), np.fft.rfftn(x.astype(np.float64))) <= 2 * c32_tolerance(x.size)
    yd = torch.empty_like(xd)
    plan.execute(yd, Xd, inverse=True)
    assert rel_rms(yd.cpu().numpy() / x.size, x) <= 4 * c32_tolerance(x.size)
    # odd last axis of a real plan is rejected like the reference
    with pytest.raises(k.KfrError, match="even"):
        k.dft_plan_md_real((4, 7))


def _oracle_fftn(orc, x, inverse=False):
    """The oracle's FP64 1-D DFT applied along every axis (a multi-dimensional DFT is separable)."""
    y = x.astype(np.complex128)
    for ax in range(y.ndim):
        moved = np.ascontiguousarray(np.moveaxis(y, ax, -1))
        y = np.moveaxis(orc.dft(moved, inverse=inverse, threads=8), -1, ax)
    return y


@pytest.mark.parametrize("shape", [(65536, 64), (30720, 3, 4), (40009, 2), (8191, 5, 6), (2, 65537, 3)])
def test_md_long_non_last_axes(orc, shape):
    """Non-last axes longer than one CTA (four-step 65536 and 30720, Bluestein 40009 and 65537, Rader 8191):
    transposed, transformed by the 1-D engine and transposed back (include/kfr/dft/fft.hpp:570-924 accepts
    any shape)."""
    rng = np.random.default_rng(sum(shape))
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    plan = k.dft_plan_md(shape)
    assert "transposed" in plan.describe()
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    plan.execute(yd, xd)
    assert rel_rms(yd.cpu().numpy(), _oracle_fftn(orc, x)) <= c32_tolerance(x.size)
    plan.execute(yd, xd, inverse=True)
    assert rel_rms(yd.cpu().numpy(), _oracle_fftn(orc, x, inverse=True)) <= c32_tolerance(x.size)
    # host buffers and the plan's own scratch
    y = np.zeros_like(x)
    plan.execute(y, x)
    assert rel_rms(y, _oracle_fftn(orc, x)) <= c32_tolerance(x.size)


def test_md_real_long_first_axis(orc):
    """A real 2-D plan whose first axis (65536) needs the transposed pass: forward against the oracle's
    per-axis transform of the real input, and the round trip."""
    shape = (65536, 16)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape).astype(np.float32)
    plan = k.dft_plan_md_real(shape)
    Xd = torch.empty(plan.complex_shape, dtype=torch.complex64, device="cuda")
    xd = torch.from_numpy(x).cuda()
    plan.execute(Xd, xd)
    full = _oracle_fftn(orc, x.astype(np.complex128))
    assert rel_rms(Xd.cpu().numpy(), full[:, : shape[1] // 2 + 1]) <= c32_tolerance(x.size)
    yd = torch.empty_like(xd)
    plan.execute(yd, Xd, inverse=True)
    assert rel_rms(yd.cpu().numpy() / x.size, x) <= 2 * c32_tolerance(x.size)  # two transforms
