"""exgb_repeat_fourier_noalloc: the stepping entry point for callers that
cannot allocate device memory where they step (for example a framework's
custom call that may only touch the buffers it is handed).  Its stage
buffers live in a fixed 8 MiB static device array instead of the plan's
allocation.  This file is collected last so that a failure here comes after
every other test has run.  The test must pass alone in a fresh process and
after the rest of the suite."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _rel(a, b):
    a = a.cpu().numpy().view(np.float32).astype(np.float64)
    b = b.cpu().numpy().view(np.float32).astype(np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("N,order", [(256, 2), (128, 4)])
def test_noalloc_matches_repeat_fourier_on_two_calls(N, order):
    import exponax_gb300 as ex
    from exponax_gb300 import _device, _lib

    lib = _lib.load()
    st = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3, order=order)
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    u0 = torch.from_numpy(np.stack([g(N, key=s) for s in range(24)])).cuda()
    uh = ex.fft(u0, num_spatial_dims=2)
    h = st.plan.handle
    ref = torch.empty_like(uh)
    _lib.check(lib.exgb_repeat_fourier(h, _device.stream(), uh.data_ptr(), ref.data_ptr(), 24, 5))
    for _ in range(2):  # the static array keeps the previous call's contents
        out = torch.full_like(uh, float("nan"))
        _lib.check(lib.exgb_repeat_fourier_noalloc(h, _device.stream(), uh.data_ptr(), out.data_ptr(), 24, 5))
        torch.cuda.synchronize()
        assert torch.isfinite(torch.view_as_real(out)).all()
        assert _rel(out, ref) < 1e-5


def test_noalloc_rejects_plans_it_cannot_serve():
    import exponax_gb300 as ex
    from exponax_gb300 import _device, _lib

    lib = _lib.load()
    st = ex.stepper.Burgers(1, 1.0, 64, 0.01)
    uh = torch.zeros((1, 1, 33), dtype=torch.complex64, device="cuda")
    rc = lib.exgb_repeat_fourier_noalloc(st.plan.handle, _device.stream(), uh.data_ptr(), uh.data_ptr(), 1, 1)
    assert rc == _lib.EXGB_EUNSUPPORTED
    assert b"2D vorticity" in lib.exgb_last_error()


def test_noalloc_refuses_a_plan_switched_to_split_bf16():
    """The entry point runs FP32 transforms only: a plan switched to the
    split-BF16 tensor-core DFT is refused instead of being stepped with other
    arithmetic than exgb_repeat_fourier uses for it."""
    import exponax_gb300 as ex
    from exponax_gb300 import _device, _lib

    lib = _lib.load()
    st = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01).set_dft_precision("split_bf16")
    uh = torch.zeros((2, 1, 128, 65), dtype=torch.complex64, device="cuda")
    rc = lib.exgb_repeat_fourier_noalloc(st.plan.handle, _device.stream(), uh.data_ptr(), uh.data_ptr(), 2, 1)
    assert rc == _lib.EXGB_EUNSUPPORTED
    assert b"split-BF16" in lib.exgb_last_error()
    st.set_dft_precision("fp32")
    out = torch.full_like(uh, float("nan"))
    _lib.check(lib.exgb_repeat_fourier_noalloc(st.plan.handle, _device.stream(), uh.data_ptr(), out.data_ptr(), 2, 1))
    torch.cuda.synchronize()
    assert torch.isfinite(torch.view_as_real(out)).all()
