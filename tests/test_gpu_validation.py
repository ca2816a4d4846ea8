"""Physics validation of the CUDA path against analytic solutions, as the reference's validation
notebooks do it (validation/validate_burgers_against_cole_hopf.ipynb,
validate_kdv_against_analytical_soliton.ipynb), all on the GPU: steppers, spectral derivative and
transforms.  Each bar is stated in the test; the float64 oracle's own error on the same case is the
yardstick (the bars leave a factor of about 2)."""

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_burgers_against_cole_hopf():
    """u = -2 nu d/dx log(phi) with phi solving the heat equation (Cole-Hopf): the GPU Burgers rollout
    against the GPU diffusion rollout mapped through the transform, notebook parameters (L = 2 pi,
    N = 100, dt = 0.01, nu = 0.001).  Float64 oracle: 2.6e-3 after 100 steps, 4.9e-4 after 1000."""
    L, N, dt, nu = 2 * np.pi, 100, 0.01, 0.001
    x = ex.make_grid(1, L, N).astype(np.float64)
    phi0 = (1.5 - (np.exp(-10 * (x - np.pi) ** 2) + 0.1)).astype(np.float32)
    u0 = (-2 * nu * o.derivative(np.log(phi0.astype(np.float64)), L)).astype(np.float32)
    burgers = ex.stepper.Burgers(1, L, N, dt, diffusivity=nu)
    heat = ex.stepper.Diffusion(1, L, N, dt, diffusivity=nu)
    for steps, bar in ((100, 5e-3), (1000, 1e-3)):
        ub = ex.repeat(burgers, steps)(torch.from_numpy(u0).cuda())
        ph = ex.repeat(heat, steps)(torch.from_numpy(phi0).cuda())
        uch = -2 * nu * ex.derivative(torch.log(ph), L)
        assert rel(ub.cpu().numpy(), uch.cpu().numpy()) < bar, steps


def test_kdv_soliton_travels_at_its_speed():
    """-c/2 sech^2(sqrt(c)/2 (x - c t - a)), c = 5, a = 10, L = 20, N = 256, dt = 1e-3 (b = -6 form, no
    hyper-diffusion): after 100 steps the GPU state is within 1 % of the translated soliton (the float64
    oracle: 0.77 %, first order in dt because the reference keeps only the real part of the
    phi-coefficients) and within 1e-5 of the float64 oracle."""
    L, N, dt, c, a = 20.0, 256, 1e-3, 5.0, 10.0
    x = ex.make_grid(1, L, N).astype(np.float64)

    def sol(t):
        return -c / 2 / np.cosh(np.sqrt(c) / 2 * (x - c * t - a)) ** 2

    st = ex.stepper.KortewegDeVries(1, L, N, dt, hyper_diffusivity=0.0)
    so = o.KortewegDeVries(1, L, N, dt, hyper_diffusivity=0.0, dtype="float64")
    u0 = sol(0.0).astype(np.float32)
    got = ex.repeat(st, 100)(torch.from_numpy(u0).cuda()).cpu().numpy()
    assert rel(got, sol(0.1)) < 1e-2
    assert rel(got, o.repeat(so, 100)(u0.astype(np.float64))) < 1e-5
