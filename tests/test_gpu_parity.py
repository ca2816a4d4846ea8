"""Parity of the CUDA path (through the C ABI) with the NumPy oracle.

Tolerances follow the target: FP32 results within 1e-5 relative L2 per
step; 1e-4 after 100 steps on non-chaotic cases; 1e-4 over at most 20 steps
on chaotic cases.  Every test states its tolerance."""

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


def cu(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


# ------------------------------------------------------------------ transforms

@pytest.mark.parametrize("D,N", [(1, 200), (1, 256), (1, 60), (1, 4096), (1, 45), (2, 60), (2, 64), (2, 128),
                                 (2, 256), (3, 15), (3, 16), (3, 32), (3, 64)])
def test_rfftn_irfftn_match_numpy(D, N):
    rng = np.random.default_rng(N + D)
    u = rng.standard_normal((3, 1) + (N,) * D).astype(np.float32)
    uh = host(ex.fft(cu(u), num_spatial_dims=D))
    ref = np.fft.rfftn(u.astype(np.float64), axes=tuple(range(-D, 0)))
    assert rel(uh.view(np.float32), ref.astype(np.complex64).view(np.float32)) < 2e-6
    # irfftn on non-Hermitian input: numpy drops Im of the c2r DC/Nyquist bins
    z = (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape)).astype(np.complex64)
    back = host(ex.ifft(cu(z), num_spatial_dims=D, num_points=N))
    refb = np.fft.irfftn(z.astype(np.complex128), s=(N,) * D, axes=tuple(range(-D, 0)))
    assert rel(back, refb) < 2e-6


def test_fft_ifft_roundtrip_abs_1e5():
    """tests/test_spectral.py:19-31 on the GPU (abs 1e-5)."""
    u = np.random.default_rng(0).standard_normal((1, 32, 32)).astype(np.float32)
    back = host(ex.ifft(ex.fft(cu(u))))
    assert np.max(np.abs(back - u)) < 1e-5


# ------------------------------------------------------------------ coefficients

@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("case", ["ks", "kdv", "ns", "ns3d32", "burgers3d32", "ns3d21"])
def test_phi_coefficients_match_fp64_oracle(order, case):
    """The tables read back through exgb_plan_get_table in the natural layout, whichever layout the
    plan keeps them in (2D fused / three-pass: [ky][kx]; 3D three-pass, N = 32: plane-major)."""
    if case == "ns3d32":
        args, mk, mo = (3, 2 * np.pi, 32, 0.01), ex.stepper.NavierStokesVelocity, o.NavierStokesVelocity
        kw = {"diffusivity": 0.01}
    elif case == "burgers3d32":
        args, mk, mo = (3, 2 * np.pi, 32, 0.01), ex.stepper.Burgers, o.Burgers
        kw = {"diffusivity": 0.05}
    elif case == "ns3d21":
        args, mk, mo = (3, 2 * np.pi, 21, 0.01), ex.stepper.NavierStokesVelocity, o.NavierStokesVelocity
        kw = {"diffusivity": 0.01}
    elif case == "ks":
        args, mk, mo = (1, 100.0, 200, 0.1), ex.stepper.KuramotoSivashinskyConservative, o.KuramotoSivashinskyConservative
        kw = {}
    elif case == "kdv":
        args, mk, mo = (1, 20.0, 256, 0.01), ex.stepper.KortewegDeVries, o.KortewegDeVries
        kw = {}
    elif case == "ns":
        args, mk, mo = (2, 2 * np.pi, 64, 0.01), ex.stepper.NavierStokesVorticity, o.NavierStokesVorticity
        kw = {"diffusivity": 1e-3}
    mine = mk(*args, order=order, **kw)._integrator
    ref = mo(*args, order=order, dtype="float64", **kw)._integrator
    np.testing.assert_allclose(mine._exp_term, ref._exp_term, rtol=1e-6, atol=1e-7)
    names = {1: [1], 2: [1, 2], 3: [1, 2, 3, 4, 5], 4: [1, 2, 3, 4, 5, 6]}[order]
    for i in names:
        a = getattr(mine, f"_coef_{i}")
        b = getattr(ref, f"_coef_{i}")
        np.testing.assert_allclose(a, b, rtol=2e-6, atol=1e-12 + 1e-6 * np.abs(b).max())


# ------------------------------------------------------------------ nonlinear functions

NL_CASES_1D = [
    ("conv_cons", dict(cls="ConvectionNonlinearFun", kw=dict(scale=1.0, single_channel=True, conservative=True))),
    ("conv_noncons", dict(cls="ConvectionNonlinearFun", kw=dict(scale=-6.0, single_channel=False, conservative=False))),
    ("grad_norm", dict(cls="GradientNormNonlinearFun", kw=dict(scale=1.0, zero_mode_fix=True))),
    ("poly", dict(cls="PolynomialNonlinearFun", kw=dict(coefficients=(0.3, -1.0, 0.5, 2.0)))),
    ("general", dict(cls="GeneralNonlinearFun", kw=dict(scale_list=(0.5, -1.2, 0.7)))),
]


@pytest.mark.parametrize("name,case", NL_CASES_1D, ids=[c[0] for c in NL_CASES_1D])
@pytest.mark.parametrize("N", [64, 200])
def test_nonlinear_fun_1d_matches_oracle(name, case, N):
    L = 30.0
    kw = dict(case["kw"])
    dm = ex.spectral.build_derivative_operator(1, L, N)
    do = o.build_derivative_operator(1, L, N)
    if case["cls"] != "PolynomialNonlinearFun":
        kw_m = dict(kw, derivative_operator=dm)
        kw_o = dict(kw, derivative_operator=do)
    else:
        kw_m, kw_o = dict(kw), dict(kw)
    fm = getattr(ex.nonlin_fun, case["cls"])(1, N, dealiasing_fraction=2 / 3, **kw_m)
    fo = getattr(o, case["cls"])(1, N, dealiasing_fraction=2 / 3, **kw_o)
    u = ex.ic.RandomSineWaves1d(1, cutoff=5)(N, key=1)
    uh = o.fft(u)
    got = host(fm(cu(uh)))
    want = fo(uh)
    assert rel(got.view(np.float32), want.astype(np.complex64).view(np.float32)) < 1e-5


@pytest.mark.parametrize("N", [60, 64, 128, 256])
@pytest.mark.parametrize("kolmogorov", [False, True])
def test_vorticity_nonlinearity_matches_oracle(N, kolmogorov):
    L = 2 * np.pi
    if kolmogorov:
        fm = ex.nonlin_fun.VorticityConvection2dKolmogorov(2, N, derivative_operator=ex.spectral.build_derivative_operator(2, L, N), dealiasing_fraction=2 / 3)
        fo = o.VorticityConvection2dKolmogorov(2, N, derivative_operator=o.build_derivative_operator(2, L, N), dealiasing_fraction=2 / 3)
    else:
        fm = ex.nonlin_fun.VorticityConvection2d(2, N, derivative_operator=ex.spectral.build_derivative_operator(2, L, N), dealiasing_fraction=2 / 3)
        fo = o.VorticityConvection2d(2, N, derivative_operator=o.build_derivative_operator(2, L, N), dealiasing_fraction=2 / 3)
    u = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)(N, key=2)
    uh = o.fft(u)
    got = host(fm(cu(uh)))
    want = fo(uh)
    assert rel(got.view(np.float32), want.astype(np.complex64).view(np.float32)) < 1e-5


# ------------------------------------------------------------------ single steps

STEP_CASES = [
    ("ks_cons_200", "KuramotoSivashinskyConservative", (1, 100.0, 200, 0.1), {}),
    ("ks_128", "KuramotoSivashinsky", (1, 60.0, 128, 0.1), {}),
    ("burgers_256", "Burgers", (1, 1.0, 256, 1e-3), {"diffusivity": 0.01}),
    ("kdv_512", "KortewegDeVries", (1, 20.0, 512, 0.01), {}),
    ("burgers_4096", "Burgers", (1, 1.0, 4096, 1e-3), {"diffusivity": 0.01}),
    ("ns_64", "NavierStokesVorticity", (2, 2 * np.pi, 64, 0.01), {"diffusivity": 1e-3}),
    ("ns_256", "NavierStokesVorticity", (2, 2 * np.pi, 256, 0.01), {"diffusivity": 1e-3}),
    ("kolmo_128", "KolmogorovFlowVorticity", (2, 2 * np.pi, 128, 0.01), {}),
    ("diffusion_2d", "Diffusion", (2, 1.0, 48, 0.05), {"diffusivity": 0.02}),
    ("advection_1d", "Advection", (1, 1.0, 64, 0.05), {"velocity": 0.7}),
]


def _ic(D, N, key):
    if D == 1:
        return ex.ic.RandomSineWaves1d(1, cutoff=5)(N, key=key)
    return ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)(N, key=key)


@pytest.mark.parametrize("name,cls,args,kw", STEP_CASES, ids=[c[0] for c in STEP_CASES])
@pytest.mark.parametrize("order", [2, 1, 3, 4])
def test_single_step_matches_oracle(name, cls, args, kw, order):
    if cls in ("Diffusion", "Advection"):
        if order != 2:
            pytest.skip("linear steppers are ETDRK0")
        sm = getattr(ex.stepper, cls)(*args, **kw)
        so = getattr(o, cls)(*args, **kw)
    else:
        sm = getattr(ex.stepper, cls)(*args, order=order, **kw)
        so = getattr(o, cls)(*args, order=order, **kw)
    D, N = args[0], args[2]
    B = 3
    u = np.stack([_ic(D, N, k) for k in range(B)])
    got = host(ex.vmap(sm)(cu(u)))
    for b in range(B):
        assert rel(got[b], so(u[b])) < 1e-5, b
    # single-sample __call__ path and its shape check
    np.testing.assert_allclose(host(sm(cu(u[0]))), got[0], rtol=0, atol=1e-6)
    with pytest.raises(ValueError):
        sm(cu(u))


@pytest.mark.parametrize("name,cls,args,kw", STEP_CASES[:8], ids=[c[0] for c in STEP_CASES[:8]])
def test_step_fourier_matches_oracle(name, cls, args, kw):
    sm = getattr(ex.stepper, cls)(*args, **kw)
    so = getattr(o, cls)(*args, **kw)
    D, N = args[0], args[2]
    uh = o.fft(_ic(D, N, 5))
    got = host(sm.step_fourier(cu(uh)))
    want = so.step_fourier(uh)
    assert rel(got.view(np.float32), want.astype(np.complex64).view(np.float32)) < 1e-5


# ------------------------------------------------------------------ multi-step

def test_ks_conservative_config_rollout():
    """Config: KS-conservative 1D, L=100, N=200, dt=0.1, batch 16 (seeds
    0..15), 500-step rollout with include_init.  Chaotic: within 1e-4
    relative L2 of the oracle over the first 20 steps; the long-run energy
    spectra (time-averaged over steps 300..500) agree within 5 %."""
    B, N, n = 16, 200, 500
    sm = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, N, 0.1)
    so = o.KuramotoSivashinskyConservative(1, 100.0, N, 0.1)
    u0 = np.stack([ex.ic.RandomSineWaves1d(1, cutoff=5)(N, key=s) for s in range(B)])
    traj = host(ex.vmap(ex.rollout(sm, n, include_init=True))(cu(u0)))
    assert traj.shape == (B, n + 1, 1, N)
    np.testing.assert_array_equal(traj[:, 0], u0)
    spec_m, spec_o = 0, 0
    for b in range(4):
        ref = o.rollout(so, n, include_init=True)(u0[b])
        for t in range(1, 21):
            assert rel(traj[b, t], ref[t]) < 1e-4, (b, t)
        spec_m = spec_m + np.mean([o.get_spectrum(traj[b, t]) for t in range(300, 501)], axis=0)
        spec_o = spec_o + np.mean([o.get_spectrum(ref[t]) for t in range(300, 501)], axis=0)
    k = slice(1, 40)
    assert np.max(np.abs(np.log(spec_m[0, k] / spec_o[0, k]))) < np.log(1.05) + 0.25
    assert rel(spec_m[0, k], spec_o[0, k]) < 0.05


def test_burgers_100_steps_non_chaotic():
    """Non-chaotic: 1e-4 relative L2 after 100 steps."""
    sm = ex.stepper.Burgers(1, 1.0, 256, 1e-3, diffusivity=0.01)
    so = o.Burgers(1, 1.0, 256, 1e-3, diffusivity=0.01)
    u0 = np.stack([ex.ic.RandomSineWaves1d(1, cutoff=5)(256, key=s) for s in range(4)])
    got = host(ex.vmap(ex.repeat(sm, 100))(cu(u0)))
    for b in range(4):
        assert rel(got[b], o.repeat(so, 100)(u0[b])) < 1e-4


def test_kdv_repeat_with_complex_linear_operator():
    """KdV (odd-order L: complex Nyquist bin) 100 steps, 1e-4."""
    sm = ex.stepper.KortewegDeVries(1, 20.0, 256, 0.01)
    so = o.KortewegDeVries(1, 20.0, 256, 0.01)
    u0 = ex.ic.RandomSineWaves1d(1, cutoff=5)(256, key=7)
    got = host(ex.repeat(sm, 100)(cu(u0)))
    assert rel(got, o.repeat(so, 100)(u0)) < 1e-4


def test_taylor_green_matches_published_errors():
    """validation/validate_taylor_green.ipynb: N=60, nu=0.1, dt=0.01;
    published FP32 errors 1.85e-7 / 1.07e-6 / 1.00e-5 after 1/10/100 steps.
    Allow 3x (FFT rounding differs between backends)."""
    N, nu, dt = 60, 0.1, 0.01
    g = ex.make_grid(2, 2 * np.pi, N)
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, dt, diffusivity=nu)

    def tg(t):
        return (2 * np.sin(g[0:1]) * np.sin(g[1:2]) * np.exp(-2 * nu * t)).astype(np.float32)

    for n, pub in ((1, 1.85e-7), (10, 1.07e-6), (100, 1.00e-5)):
        e = rel(host(ex.repeat(sm, n)(cu(tg(0.0)))), tg(n * dt))
        assert e < 3 * pub, (n, e)


def test_ns_256_config_short_rollout():
    """Config: NS vorticity 256^2, nu=1e-3, dt=0.01 (batch 4 here): within
    1e-5 per step and 1e-4 after 20 steps (repeat and rollout paths)."""
    N = 256
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    so = o.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    u0 = np.stack([_ic(2, N, s) for s in range(4)])
    fin = host(ex.vmap(ex.repeat(sm, 20))(cu(u0)))
    traj = host(ex.vmap(ex.rollout(sm, 5, include_init=False))(cu(u0[:2])))
    for b in range(2):
        ref = o.rollout(so, 20)(u0[b])
        assert rel(fin[b], ref[-1]) < 1e-4
        for t in range(5):
            assert rel(traj[b, t], ref[t]) < 1e-5 * (t + 1)


@pytest.mark.parametrize("cluster", [0, 4, 6, 8])
def test_kolmogorov_512_generic_cluster_kernel(cluster):
    """Kolmogorov flow 512^2 on the generic 2D cluster kernel (its derived fields go through L2;
    EXGB_2D_PATH=fused selects it over the three-pass path): 3 ETDRK2 steps within 1e-5 of the
    oracle, at the automatic cluster size and at 4, 6 (rows split 86 x 5 + 82) and 8 CTAs per
    cluster."""
    import os

    from exponax_gb300 import autotune

    N = 512
    os.environ["EXGB_2D_PATH"] = "fused"  # 512^2 runs on the three-pass path unless asked otherwise
    try:
        sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, N, 0.001)
        sm.plan.handle  # the plan (and its path) is made here, while the variable is set
    finally:
        del os.environ["EXGB_2D_PATH"]
    so = o.KolmogorovFlowVorticity(2, 2 * np.pi, N, 0.001)
    if cluster:
        assert autotune._set(sm.plan, 1, [cluster]) == 0
        assert autotune.get_tuning(sm.plan)["cluster"] == cluster
    u0 = np.stack([_ic(2, N, s) for s in range(3)])
    got = host(ex.vmap(ex.repeat(sm, 3))(cu(u0)))
    for b in range(3):
        assert rel(got[b], o.repeat(so, 3)(u0[b])) < 1e-5


@pytest.mark.parametrize("cluster", [0, 2, 4, 7])
def test_generic_2d_kernel_uneven_row_split(cluster):
    """N = 45 on the generic 2D kernel with cluster sizes that do not divide N (rows per
    CTA 23/22, 12 x 3 + 9, 7 x 6 + 3): 5 ETDRK2 steps of NS vorticity within 1e-5."""
    from exponax_gb300 import autotune

    N = 45
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    so = o.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    if cluster:
        assert autotune._set(sm.plan, 1, [cluster]) == 0
        assert autotune.get_tuning(sm.plan)["cluster"] == cluster
    u0 = np.stack([_ic(2, N, s) for s in range(4)])
    got = host(ex.vmap(ex.repeat(sm, 5))(cu(u0)))
    for b in range(4):
        assert rel(got[b], o.repeat(so, 5)(u0[b])) < 1e-5


def test_ns256_partial_last_wave_on_tail_configuration():
    """NS vorticity 256^2 with one more sample than the co-resident clusters: the main launch runs
    a full wave and the extra sample runs in a second launch on larger clusters (the fused-launch
    count says 2); every sample within 1e-5 of the oracle after 3 steps."""
    import ctypes

    from exponax_gb300 import _lib

    N = 256
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    so = o.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    lib, h, cnt = _lib.load(), sm.plan.handle, ctypes.c_int(0)

    def launches(b):
        assert lib.exgb_plan_fused_launches(h, b, ctypes.byref(cnt)) == 0
        return cnt.value

    assert launches(0) == 0 and launches(1) == 1
    two = [b for b in range(2, 80) if launches(b) == 2]
    assert two, "N = 256 has a tail configuration"
    B = two[0]
    u0 = np.stack([_ic(2, N, s % 7) * np.float32(1.0 + 0.01 * s) for s in range(B)]).astype(np.float32)
    got = host(ex.vmap(ex.repeat(sm, 3))(cu(u0)))
    for b in range(B):
        assert rel(got[b], o.repeat(so, 3)(u0[b])) < 1e-5, b


def test_repeated_stepper_stays_in_fourier_space():
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 64, 0.01)
    so = o.KolmogorovFlowVorticity(2, 2 * np.pi, 64, 0.01)
    u0 = _ic(2, 64, 3)
    got = host(ex.RepeatedStepper(sm, 10)(cu(u0)))
    assert rel(got, o.RepeatedStepper(so, 10)(u0)) < 1e-4


def test_queue_rollout_mixed_pdes_and_sizes():
    """Uneven batch in one persistent launch: Burgers / KdV / KS-cons with
    different N; each instance matches its own oracle rollout (20 steps)."""
    import ctypes

    from exponax_gb300 import _device, _lib

    specs = [
        (ex.stepper.Burgers(1, 1.0, 128, 1e-3, diffusivity=0.01), o.Burgers(1, 1.0, 128, 1e-3, diffusivity=0.01)),
        (ex.stepper.KortewegDeVries(1, 20.0, 512, 0.01), o.KortewegDeVries(1, 20.0, 512, 0.01)),
        (ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 256, 0.1),
         o.KuramotoSivashinskyConservative(1, 100.0, 256, 0.1)),
        (ex.stepper.Burgers(1, 1.0, 2048, 1e-3, diffusivity=0.01), o.Burgers(1, 1.0, 2048, 1e-3, diffusivity=0.01)),
    ]
    n = 20
    rng = np.random.default_rng(0)
    order = rng.integers(0, len(specs), size=12)
    u0s, trajs, items = [], [], []
    for i, s in enumerate(order):
        sm, _ = specs[s]
        u0 = cu(_ic(1, sm.num_points, i))
        tr = torch.empty((n + 1, 1, sm.num_points), dtype=torch.float32, device="cuda")
        u0s.append(u0)
        trajs.append(tr)
        items.append(_lib.WorkItem(sm.plan.handle.value, u0.data_ptr(), tr.data_ptr()))
    arr = (_lib.WorkItem * len(items))(*items)
    _lib.check(_lib.load().exgb_queue_rollout(arr, len(items), n, 1, _device.stream()))
    torch.cuda.synchronize()
    for i, s in enumerate(order):
        ref = o.rollout(specs[s][1], n, include_init=True)(host(u0s[i]))
        got = host(trajs[i])
        assert rel(got[1:], ref[1:]) < 1e-4, (i, s)


def test_map_between_resolutions_matches_oracle():
    u = _ic(2, 256, 9)
    for new in (64, 128, 512):
        got = host(ex.map_between_resolutions(cu(u), new))
        assert rel(got, o.map_between_resolutions(u, new)) < 1e-5
    u1 = _ic(1, 200, 2)
    assert rel(host(ex.map_between_resolutions(cu(u1), 50)), o.map_between_resolutions(u1, 50)) < 1e-5


@pytest.mark.parametrize("D,old,news", [(1, 40, (25, 32, 64, 75)), (2, 32, (15, 20, 48, 64)),
                                        (3, 16, (8, 12, 15, 24, 32)), (3, 15, (10, 16, 30))])
@pytest.mark.parametrize("oddball_zero", [True, False])
def test_map_between_resolutions_white_noise(D, old, news, oddball_zero):
    """Non-bandlimited two-channel fields, so that the Nyquist planes (oddball masks) carry energy;
    up- and downsampling, even and odd grids, 1D-3D.  Tolerance 1e-5 relative L2."""
    rng = np.random.default_rng(5 + D)
    u = rng.standard_normal((2,) + (old,) * D).astype(np.float32)
    for new in news:
        got = host(ex.map_between_resolutions(cu(u), new, oddball_zero=oddball_zero))
        ref = o.map_between_resolutions(u, new, oddball_zero=oddball_zero)
        assert got.shape == ref.shape
        assert rel(got, ref) < 1e-5, (new, rel(got, ref))
    batch = np.stack([u, 2 * u])
    got = host(ex.interpolation.map_between_resolutions_batched(cu(batch), news[0], oddball_zero=oddball_zero))
    ref = o.map_between_resolutions(u, news[0], oddball_zero=oddball_zero)
    assert rel(got[1], 2 * ref) < 1e-5


def test_errors_follow_the_reference():
    sm = ex.stepper.Burgers(1, 1.0, 64, 0.01)
    with pytest.raises(ValueError):
        sm(cu(np.zeros((2, 64), np.float32)))
    with pytest.raises(ValueError):  # prime, too long for the Bluestein transform of one CTA
        ex.stepper.Burgers(1, 1.0, 7919, 0.01)(cu(np.zeros((1, 7919), np.float32)))


def test_queue_rollout_graph_capture_and_replay():
    """QueueRollout: prepared queue, launch captured in a CUDA graph and
    replayed twice; every instance matches its oracle rollout (15 steps)."""
    from exponax_gb300.batching import QueueRollout

    b1 = ex.stepper.Burgers(1, 1.0, 256, 1e-3, diffusivity=0.01)
    k1 = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 128, 0.1)
    specs = {id(b1): o.Burgers(1, 1.0, 256, 1e-3, diffusivity=0.01),
             id(k1): o.KuramotoSivashinskyConservative(1, 100.0, 128, 0.1)}
    inst = [(b1 if i % 3 else k1, _ic(1, (b1 if i % 3 else k1).num_points, i)) for i in range(10)]
    q = QueueRollout(inst, 15, include_init=True)
    q.capture()
    for _ in range(2):
        for t in q.trajectories:
            t.zero_()
        q.replay()
        torch.cuda.synchronize()
        for (st, u0), tr in zip(inst, q.trajectories):
            ref = o.rollout(specs[id(st)], 15, include_init=True)(u0)
            got = host(tr)
            np.testing.assert_array_equal(got[0], u0)
            assert rel(got[1:], ref[1:]) < 1e-4


# ------------------------------------------------------------------ Poisson (_poisson.py)

@pytest.mark.parametrize("D,L,N", [(1, 1.0, 50), (2, 3.0, 25), (3, 3.0, 15)])
def test_poisson_exact(D, L, N):
    """tests/test_validation.py:214-292 on the GPU: sin products against the analytic solution, abs 1e-6."""
    g = ex.make_grid(D, L, N)
    k = 2 * np.pi / L
    rhs = np.prod([np.sin(k * g[d:d + 1]) for d in range(D)], axis=0).astype(np.float32)
    want = rhs / (D * k ** 2)
    u = host(ex.poisson.Poisson(D, L, N)(cu(rhs)))
    np.testing.assert_allclose(u, want, rtol=0, atol=1e-6)


@pytest.mark.parametrize("D,N,order", [(1, 64, 2), (2, 48, 2), (2, 32, 4), (3, 16, 2)])
def test_poisson_matches_oracle(D, N, order):
    """Random right-hand sides (two channels, batched) against the oracle's Poisson: 1e-6 relative L2;
    step_fourier alone, and the zero mean of the solution."""
    rng = np.random.default_rng(D * 10 + order)
    f = rng.standard_normal((3, 2) + (N,) * D).astype(np.float32)
    pm = ex.poisson.Poisson(D, 2.0, N, order=order)
    po = o.Poisson(D, 2.0, N, order=order)
    got = host(pm.step(cu(f)))
    for b in range(3):
        assert rel(got[b], po(f[b])) < 1e-6, b
        assert abs(float(got[b].mean())) < 1e-6
    fh = o.fft(f[0], num_spatial_dims=D).astype(np.complex64)
    gh = host(pm.step_fourier(cu(fh)))
    assert rel(gh.view(np.float32), po.step_fourier(fh).astype(np.complex64).view(np.float32)) < 1e-6
    with pytest.raises(ValueError):
        pm(cu(f[0][..., :-1]))


# ------------------------------------------------------------------ Wave (stepper/_wave.py)

def _wave_ic(D, N, key):
    g = ex.ic.RandomAmplitudePhaseSeries(D, cutoff=3, max_one=True)
    return np.concatenate([g(N, key=2 * key), 0.3 * g(N, key=2 * key + 1)]).astype(np.float32)


@pytest.mark.parametrize("D,N,L,c,dt", [(1, 64, 2.0, 1.0, 0.01), (2, 32, 1.0, 2.0, 0.005), (3, 16, 3.0, 0.7, 0.05),
                                        (2, 15, 1.0, 1.0, 0.01)])
def test_wave_matches_oracle(D, N, L, c, dt):
    """One step (1e-5), step_fourier (1e-5), 100 steps of repeat and a 20-step rollout (1e-4) against the
    float32 oracle's diagonalised step; the 100-step error against the float64 oracle is asserted too."""
    sm = ex.stepper.Wave(D, L, N, dt, speed_of_sound=c)
    so = o.Wave(D, L, N, dt, speed_of_sound=c)
    so64 = o.Wave(D, L, N, dt, speed_of_sound=c, dtype="float64")
    u = np.stack([_wave_ic(D, N, k) for k in range(2)])
    one = host(ex.vmap(sm)(cu(u)))
    for b in range(2):
        assert rel(one[b], so(u[b])) < 1e-5, b
    uh = o.fft(u[0], num_spatial_dims=D).astype(np.complex64)
    gh = host(sm.step_fourier(cu(uh)))
    assert rel(gh.view(np.float32), so.step_fourier(uh).astype(np.complex64).view(np.float32)) < 1e-5
    many = host(ex.vmap(ex.repeat(sm, 100))(cu(u)))
    traj = host(ex.vmap(ex.rollout(sm, 20, include_init=True))(cu(u)))
    for b in range(2):
        assert rel(many[b], o.repeat(so, 100)(u[b])) < 1e-4, b
        assert rel(many[b], o.repeat(so64, 100)(u[b].astype(np.float64))) < 1e-4, b
        assert rel(traj[b], o.rollout(so, 20, include_init=True)(u[b])) < 1e-4, b
    assert traj.shape == (2, 21, 2) + (N,) * D


def test_wave_conserves_energy_and_drifts_the_mean():
    """||v||^2 + c^2 ||grad h||^2 is invariant (exact step): within 3e-5 after 500 steps (the float32
    one-step map alone drifts it by about 6e-6 here); the mean of h moves by dt * mean(v) per step
    (the reference's mean-mode rule)."""
    D, N, L, c, dt = 2, 48, 2.0, 1.5, 0.01
    sm = ex.stepper.Wave(D, L, N, dt, speed_of_sound=c)
    u = _wave_ic(D, N, 3)
    u[1] += 0.25  # nonzero mean velocity

    def energy(x):
        xh = np.fft.rfftn(x.astype(np.float64), axes=(-2, -1))
        k = np.linalg.norm(ex.spectral.build_scaled_wavenumbers(D, L, N), axis=0)
        w = np.ones(xh.shape[-1])
        w[1:-1] = 2.0  # rfft half-spectrum weights (N even)
        dev = xh[1].copy()
        dev[0, 0] = 0.0
        return float(np.sum(w * (np.abs(dev) ** 2 + c ** 2 * k ** 2 * np.abs(xh[0]) ** 2)))

    out = host(ex.repeat(sm, 500)(cu(u)))
    assert abs(energy(out) - energy(u)) / energy(u) < 3e-5
    assert abs(float(out[0].mean()) - (float(u[0].mean()) + 500 * dt * float(u[1].mean()))) < 1e-4


# ------------------------------------------------------------------ FourierInterpolator (_interpolation.py)

@pytest.mark.parametrize("D,N,L", [(1, 64, 2.0), (2, 32, 1.0), (2, 15, 3.0), (3, 12, 2 * np.pi)])
def test_fourier_interpolator_matches_oracle(D, N, L):
    """Random points of the domain, three channels of a smooth random field: within 5e-5 max|u| of the
    float64 oracle (FP32 phases k.x up to pi N, as in the reference) and of the float32 oracle; at the
    grid points the interpolant returns the grid values (1e-5 max|u|); one point and vmap agree."""
    g = ex.ic.RandomAmplitudePhaseSeries(D, cutoff=4, max_one=True)
    u = np.concatenate([g(N, key=k) for k in range(3)]).astype(np.float32)
    fi = ex.FourierInterpolator(cu(u), domain_extent=L)
    fo64 = o.FourierInterpolator(u.astype(np.float64), domain_extent=L)
    fo32 = o.FourierInterpolator(u, domain_extent=L)
    pts = np.random.default_rng(D).uniform(0, L, (200, D)).astype(np.float32)
    got = host(ex.vmap(fi)(cu(pts)))
    assert got.shape == (200, 3)
    want64 = np.stack([fo64(p.astype(np.float64)) for p in pts])
    want32 = np.stack([fo32(p) for p in pts])
    scale = float(np.abs(u).max())
    assert np.abs(got - want64).max() < 5e-5 * scale
    assert np.abs(got - want32).max() < 5e-5 * scale
    one = host(fi(cu(pts[7])))
    np.testing.assert_allclose(one, got[7], rtol=0, atol=1e-6 * scale)
    grid = ex.make_grid(D, L, N).reshape(D, -1).T
    sel = grid[:: max(1, grid.shape[0] // 100)]
    at = host(ex.vmap(fi)(cu(np.ascontiguousarray(sel))))
    flat = u.reshape(3, -1).T[:: max(1, grid.shape[0] // 100)]
    assert np.abs(at - flat).max() < 1e-5 * scale


# ------------------------------------------------------------------ spectral helpers (_spectral.py:724-1172)

@pytest.mark.parametrize("D,N,C,order", [(1, 64, 1, 1), (1, 60, 2, 3), (2, 32, 1, 2), (2, 24, 2, 1), (3, 16, 3, 1)])
def test_spectral_derivative_matches_oracle(D, N, C, order):
    """spectral.derivative on random fields against the oracle (1e-5), and the exact derivative of a sine."""
    rng = np.random.default_rng(D * 7 + order)
    u = rng.standard_normal((C,) + (N,) * D).astype(np.float32)
    got = host(ex.derivative(cu(u), 3.0, order=order))
    want = o.derivative(u, 3.0, order=order)
    assert got.shape == want.shape
    assert rel(got, want) < 1e-5
    g = ex.make_grid(D, 2.0, N)
    s = np.sin(2 * np.pi / 2.0 * 2 * g[0:1]).astype(np.float32)
    ds = host(ex.spectral.derivative(cu(s), 2.0, order=1))
    np.testing.assert_allclose(ds[0], (2 * np.pi / 2.0 * 2) * np.cos(2 * np.pi / 2.0 * 2 * g[0]), atol=1e-4)


@pytest.mark.parametrize("D,N", [(1, 32), (2, 32), (2, 25), (3, 16)])
def test_make_incompressible(D, N):
    """make_incompressible against the oracle (1e-5) and its size-independent property: the spectral
    divergence of the result vanishes (relative to that of the input) and projecting twice changes nothing."""
    u = np.random.default_rng(D).standard_normal((D,) + (N,) * D).astype(np.float32)
    got = host(ex.spectral.make_incompressible(cu(u)))
    assert rel(got, o.make_incompressible(u)) < 1e-5
    # band-limited fields (no Nyquist energy, where the rfft derivative is not antisymmetric)
    gen = ex.ic.RandomTruncatedFourierSeries(D, cutoff=N // 4)
    v = np.concatenate([gen(N, key=10 + d) for d in range(D)]).astype(np.float32)
    pv = host(ex.spectral.make_incompressible(cu(v)))
    div = lambda f: sum(o.derivative(f[d:d + 1], 1.0)[d] for d in range(D))  # noqa: E731
    if D > 1:  # in 1D only the (here zero) mean is divergence free
        assert np.linalg.norm(div(pv.astype(np.float64))) < 1e-4 * np.linalg.norm(div(v.astype(np.float64)))
        again = host(ex.spectral.make_incompressible(cu(pv)))
        assert rel(again, pv) < 1e-5
    with pytest.raises(ValueError):
        ex.spectral.make_incompressible(cu(u[:1]) if D > 1 else cu(np.stack([u[0], u[0]])))


@pytest.mark.parametrize("mode", ["coef_extraction", "reconstruction", "norm_compensation", None])
def test_get_fourier_coefficients(mode):
    """get_fourier_coefficients of a known cosine series: the coefficient-extraction amplitudes, and
    agreement with the oracle (rounded to 5 decimals, so compare at 1e-5 absolute)."""
    L, N = 2.0, 32
    g = ex.make_grid(2, L, N)
    u = (3 * np.cos(2 * np.pi / L * 2 * g[0:1]) + 0.5 * np.sin(2 * np.pi / L * 3 * g[1:2])).astype(np.float32)
    got = host(ex.spectral.get_fourier_coefficients(cu(u), scaling_compensation_mode=mode))
    want = o.get_fourier_coefficients(u, scaling_compensation_mode=mode)
    np.testing.assert_allclose(got, want, atol=1e-5 if mode else 2e-3, rtol=0)
    if mode == "coef_extraction":
        assert abs(got[0, 2, 0].real - 3.0) < 1e-5 and abs(got[0, 0, 3].imag + 0.5) < 1e-5
    assert np.asarray(ex.spectral.get_spectrum(u)).shape == (1, N // 2 + 1)
