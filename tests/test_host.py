"""CPU-only checks of the boundary and host logic: the C ABI library loads
and exports every declared symbol, the ctypes mirror of exgb_plan_desc
matches the C layout, and host-side operator assembly matches the oracle."""

import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import exponax_gb300 as ex
from exponax_gb300 import _lib
from oracle import exponax_np as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "exgb.h")


CORRECTOR_HEADER = os.path.join(ROOT, "include", "exgb_corrector.h")


def _declared_functions(header=HEADER):
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(exgb_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = _declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert {s[0] for s in _lib.SIGNATURES} == set(names)


def test_library_exports_every_corrector_symbol():
    from exponax_gb300.learned import CORRECTOR_SIGNATURES

    lib = _lib.load()
    names = _declared_functions(CORRECTOR_HEADER)
    for n in names:
        assert hasattr(lib, n), n
    assert set(CORRECTOR_SIGNATURES) == set(names)
    assert not set(names) & set(_declared_functions())


def test_corrector_headers_compile_together_as_c():
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(f'#include "{HEADER}"\n#include "{CORRECTOR_HEADER}"\nint main(void){{return 0;}}\n')
        subprocess.run(["gcc", "-Wall", "-Werror", c, "-o", os.path.join(d, "t")], check=True)


def test_corrector_null_arguments_are_rejected_without_touching_the_gpu():
    from exponax_gb300.learned import _lib as corr_lib

    lib = corr_lib()
    assert lib.exgb_conv_in1(None, None, 1, 64, None, None, None, None) == _lib.EXGB_EINVAL
    assert lib.exgb_conv_out1(None, None, 1, 64, None, None, None, 1.0, None) == _lib.EXGB_EINVAL
    assert lib.exgb_conv48(None, None, 1, 63, None, None, 0, None, None, None) == _lib.EXGB_EINVAL
    assert lib.exgb_wgrad(None, 3, None, None, 1, 64, None, None, None, None) == _lib.EXGB_EINVAL
    assert lib.exgb_adam(None, None, None, None, None, 10, 1e-3, 0.9, 0.999, 1e-8, 1, None, None, 0) == _lib.EXGB_EINVAL
    assert lib.exgb_cast_weights(None, None, 10, None, None, 1) == _lib.EXGB_EINVAL  # w NULL
    assert lib.exgb_mse(None, None, None, 10, 1.0, None, None, 0) == _lib.EXGB_EINVAL
    assert lib.exgb_guard(None, None, None, 1, 64, 8, 0.1, None, None, None) == _lib.EXGB_EINVAL
    assert b"NULL" in lib.exgb_last_error() or b"bad" in lib.exgb_last_error()


def test_version_and_error_string_without_gpu():
    lib = _lib.load()
    assert lib.exgb_version() == 1
    assert isinstance(lib.exgb_last_error(), bytes)


def test_null_arguments_are_rejected_without_touching_the_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.exgb_plan_create(None, ctypes.byref(h)) == _lib.EXGB_EINVAL
    assert lib.exgb_rfftn(None, 1, 16, 1, None, None) == _lib.EXGB_EINVAL
    assert b"NULL" in lib.exgb_last_error()
    d = _lib.PlanDesc()
    d.num_spatial_dims = 1
    d.num_points = 1
    d.order = 2
    d.num_channels = 1
    assert lib.exgb_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.EXGB_EINVAL
    d.num_points = 7919  # prime, too long for the Bluestein transform of one CTA
    assert lib.exgb_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.EXGB_ENOTFACTORABLE
    d.num_points = 16
    d.order = 5
    assert lib.exgb_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.EXGB_ENOTIMPL
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.EXGB_ENOTIMPL)
    with pytest.raises(ValueError):
        _lib.check(_lib.EXGB_ESHAPE)


def test_plan_desc_layout_matches_c_header():
    fields = [f[0] for f in _lib.PlanDesc._fields_]
    prog = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){"]
    prog.append('printf("%zu\\n", sizeof(exgb_plan_desc));')
    for f in fields:
        prog.append(f'printf("%zu\\n", offsetof(exgb_plan_desc, {f}));')
    prog.append('printf("%zu\\n", sizeof(exgb_work_item));')
    prog.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write("\n".join(prog))
        subprocess.run(["gcc", c, "-o", exe], check=True)
        vals = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(_lib.PlanDesc)
    for f, off in zip(fields, vals[1:-1]):
        assert getattr(_lib.PlanDesc, f).offset == off, f
    assert vals[-1] == ctypes.sizeof(_lib.WorkItem)


@pytest.mark.parametrize("cls,args,kw", [
    ("KuramotoSivashinskyConservative", (1, 100.0, 200, 0.1), {}),
    ("KuramotoSivashinsky", (1, 60.0, 128, 0.1), {}),
    ("Burgers", (1, 1.0, 256, 1e-3), {"diffusivity": 0.01}),
    ("KortewegDeVries", (1, 20.0, 512, 0.01), {"dispersivity": 1.0, "hyper_diffusivity": 0.01}),
    ("NavierStokesVorticity", (2, 2 * np.pi, 64, 0.01), {"diffusivity": 1e-3}),
    ("KolmogorovFlowVorticity", (2, 2 * np.pi, 64, 0.01), {}),
    ("Advection", (1, 1.0, 32, 0.1), {"velocity": 0.3}),
    ("Diffusion", (2, 1.0, 32, 0.1), {"diffusivity": 0.02}),
    ("Dispersion", (1, 1.0, 32, 0.1), {}),
    ("HyperDiffusion", (1, 1.0, 32, 0.1), {}),
    ("NavierStokesVelocity", (3, 2 * np.pi, 16, 0.01), {"diffusivity": 0.01}),
    ("KolmogorovFlowVelocity", (3, 2 * np.pi, 16, 0.01), {}),
    ("Diffusion", (3, 1.0, 16, 0.1), {"diffusivity": 0.02}),
])
def test_host_linear_operator_matches_oracle(cls, args, kw):
    mine = getattr(ex.stepper, cls)(*args, **kw)
    ref = getattr(o, cls)(*args, dtype="float64", **kw)
    np.testing.assert_allclose(mine.linear_operator, ref.linear_operator, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("N", [60, 64, 96, 128, 200, 256, 512, 4096])
def test_dealias_kmax_matches_oracle_mask(N):
    nf = o.BaseNonlinearFun(1, N, dealiasing_fraction=2 / 3)
    assert ex.spectral.dealias_kmax(2 / 3, N) == int(np.nonzero(nf.dealiasing_mask[0])[0].max())
    mine = ex.nonlin_fun.BaseNonlinearFun(2, N, dealiasing_fraction=2 / 3).dealiasing_mask
    np.testing.assert_array_equal(mine, o.BaseNonlinearFun(2, N, dealiasing_fraction=2 / 3).dealiasing_mask)


def test_scaling_arrays_and_slices_match_oracle():
    for D in (1, 2, 3):
        for N in (10, 11):
            for mode in ("norm_compensation", "reconstruction", "coef_extraction"):
                np.testing.assert_array_equal(ex.spectral.build_scaling_array(D, N, mode=mode),
                                              o.build_scaling_array(D, N, mode=mode, dtype="float64"))
            assert ex.spectral.get_modes_slices(D, N) == o.get_modes_slices(D, N)


def test_kolmogorov_injection_host_array():
    st = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 32, 0.01)
    ref = o.KolmogorovFlowVorticity(2, 2 * np.pi, 32, 0.01, dtype="float64")
    np.testing.assert_array_equal(st.nonlinear_fun.injection, ref.nonlinear_fun.injection)


def test_reference_errors_raised_at_construction():
    with pytest.raises(ValueError, match="2"):
        ex.stepper.NavierStokesVorticity(3, 1.0, 16, 0.1)
    with pytest.raises(NotImplementedError):
        ex.stepper.Burgers(1, 1.0, 16, 0.1, order=5)


def test_ic_generators_are_seeded_and_normalised():
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    a = g(64, key=3)
    b = g(64, key=3)
    np.testing.assert_array_equal(a, b)
    assert a.shape == (1, 64, 64)
    assert abs(np.abs(a).max() - 1) < 1e-6
    assert abs(a.mean()) < 1e-6
    s = ex.ic.RandomSineWaves1d(1, cutoff=5)(200, key=0)
    spec = np.abs(np.fft.rfft(s[0]))
    assert np.all(spec[6:] < 1e-3 * spec.max())


def test_instantiate_linear_and_wave_steppers_without_a_gpu():
    """tests/test_builtin_solvers.py:8-30: the linear steppers and Wave construct in 1D-3D on the host
    (operators only; the device plan is made on first use).  Wave's exact one-step map is the identity
    plus dt v at the mean mode and has unit determinant elsewhere."""
    for D in (1, 2, 3):
        for cls in (ex.stepper.Advection, ex.stepper.Diffusion, ex.stepper.AdvectionDiffusion,
                    ex.stepper.Dispersion, ex.stepper.HyperDiffusion, ex.stepper.Wave):
            cls(D, 10.0, 25, 0.1)
    w = ex.stepper.Wave(2, 10.0, 25, 0.1, speed_of_sound=2.0)
    m = w._mix.astype(np.float64)
    np.testing.assert_allclose(m[:, 0], [1.0, 0.1, 0.0, 1.0])
    np.testing.assert_allclose(m[0] * m[3] - m[1] * m[2], 1.0, atol=1e-6)



def test_wrap_bc_and_sub_trajectories():
    """_utils.py:65-89 and :257-313 against the oracle (host arrays), with a dict of trajectories."""
    u = np.random.default_rng(0).standard_normal((2, 5, 4, 4)).astype(np.float32)
    np.testing.assert_array_equal(ex.wrap_bc(u[0]), o.wrap_bc(u[0]))
    assert ex.wrap_bc(u[0]).shape == (5, 5, 5)
    trj = np.random.default_rng(1).standard_normal((7, 1, 8)).astype(np.float32)
    np.testing.assert_array_equal(ex.stack_sub_trajectories(trj, 3), o.stack_sub_trajectories(trj, 3))
    d = ex.stack_sub_trajectories({"u": trj, "v": (trj, 2 * trj)}, 4)
    assert d["u"].shape == (4, 4, 1, 8) and d["v"][1].shape == (4, 4, 1, 8)
    with pytest.raises(ValueError):
        ex.stack_sub_trajectories(trj, 8)
    with pytest.raises(ValueError):
        ex.stack_sub_trajectories({"a": trj, "b": trj[:5]}, 2)
