"""The library's MEX gateways (``comp_ui_toolbox_gb300/mex/``), compiled and run outside MATLAB.

Each gateway is compiled with gcc against ``oracle/ref_mex/mex.h`` and linked with that
directory's host MEX runtime (``mex_stub.cpp``) and ``libcui_born.so``; the tests build the
``operator_born`` object the gateway reads with :class:`oracle.ref_runner.ReferenceGateway`.

* CPU: the argument checks and their error identifiers, which follow the reference's gateway
  (``+scattering/combined_quick_gpu.cu:201-441``), raised before any device call.
* GPU: ``cui_born_mex(op, 1 | 2, x)`` against the reference's own outputs
  (``tests/golden/reference_gateway.npz``) and the FP64 oracle, relative L2 <= 1e-5 per column;
  the cached plan is reused for the same operator and rebuilt for a changed one or a wider
  batch; ``cui_lasso_mex`` against the library's device LASSO.
"""

from __future__ import annotations

import dataclasses
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import adjoint_quick_cpu, configs, forward_quick_cpu
from oracle.ref_runner import ReferenceGateway, RefMexError
from tests.golden.make_reference_golden import OUT
from tests.helpers import rel_l2

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "comp_ui_toolbox_gb300"
STUB = ROOT / "oracle" / "ref_mex"
BUILD = PKG / "_build" / "mex"
TOL = 1e-5


def build_gateway(name: str) -> Path:
    """lib<name>.so: the gateway plus the host MEX runtime, linked against libcui_born.so."""
    from comp_ui_toolbox_gb300 import build
    build.build()
    BUILD.mkdir(parents=True, exist_ok=True)
    cc, cxx = shutil.which("gcc") or "cc", shutil.which("g++") or "c++"
    obj, stub, lib = BUILD / f"{name}.o", BUILD / f"{name}_mex_stub.o", BUILD / f"lib{name}.so"
    for cmd in ([cc, "-std=c99", "-O1", "-fPIC", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", f"-I{STUB}",
                 "-c", str(PKG / "mex" / f"{name}.c"), "-o", str(obj)],
                [cxx, "-std=c++17", "-O1", "-fPIC", f"-I{STUB}", "-c", str(STUB / "mex_stub.cpp"), "-o", str(stub)],
                [cxx, "-shared", "-Wl,-Bsymbolic", "-o", str(lib), str(obj), str(stub), f"-L{PKG}", "-lcui_born",
                 f"-Wl,-rpath,{PKG}"]):
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
    return lib


@pytest.fixture(scope="module")
def born_mex():
    return ReferenceGateway(build_gateway("cui_born_mex"))


@pytest.fixture(scope="module")
def lasso_mex():
    return ReferenceGateway(build_gateway("cui_lasso_mex"))


def built(name):
    return configs.build(configs.small_config(name))


def test_gateways_compile_warning_free(born_mex, lasso_mex):
    assert hasattr(born_mex.lib, "mexFunction") and hasattr(lasso_mex.lib, "mexFunction")


def test_argument_errors_before_any_device_call(born_mex):
    b = built("c1")
    gw = born_mex
    node = gw.operator(b.op)
    g = configs.make_gamma(b.cfg)
    for args, ident in [((node, 3, g), "combined_quick_gpu:NoNumericScalarMode"),
                        ((node, 1j, g), "combined_quick_gpu:NoNumericScalarMode"),
                        ((node, np.array([1.0, 2.0]), g), "combined_quick_gpu:NoNumericScalarMode"),
                        ((gw.obj("scattering.operator"), 1, g), "combined_quick_gpu:NoOperatorBorn"),
                        ((gw.operator(b.op, setup_class="scattering.sequences.setups.setup"), 1, g),
                         "combined_quick_gpu:NoSymmetricGridsSetup"),
                        ((gw.operator(b.op, gpu_class="scattering.options.gpu_off"), 1, g),
                         "combined_quick_gpu:NoScatteringOptionsGPUActive")]:
        with pytest.raises(RefMexError) as ei:
            gw.call(*args)
        assert ei.value.ident == ident
    with pytest.raises(RefMexError) as ei:
        gw.call(node, 1, g, nrhs=2)
    assert ei.value.ident == "combined_quick_gpu:NumberArguments"
    gw.reset()


def test_lasso_gateway_argument_count(lasso_mex):
    b = built("c1")
    node = lasso_mex.operator(b.op)
    with pytest.raises(RefMexError) as ei:
        lasso_mex.call(node, 1, configs.make_gamma(b.cfg))  # 3 of its 6 inputs
    assert ei.value.ident == "combined_quick_gpu:NumberArguments"
    lasso_mex.reset()


# ------------------------------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "c2", "ragged", "c3"])
def test_born_mex_matches_reference_outputs(born_mex, name):
    fix = np.load(OUT)
    b = built(name)
    gw = born_mex
    node = gw.operator(b.op)
    for gk, uk in (("gamma", "u"), ("gamma_real", "u_real")):
        u = gw.call(node, 1, fix[f"{name}/{gk}"])
        assert u.shape == fix[f"{name}/{uk}"].shape
        u_or = forward_quick_cpu(b.op, fix[f"{name}/{gk}"])
        for k in range(u.shape[1]):
            assert rel_l2(u[:, k], fix[f"{name}/{uk}"][:, k]) <= TOL
            assert rel_l2(u[:, k], u_or[:, k]) <= TOL
    g = gw.call(node, 2, fix[f"{name}/y"])
    g_ref = adjoint_quick_cpu(b.op, fix[f"{name}/y"])
    for k in range(g.shape[1]):
        assert rel_l2(g[:, k], fix[f"{name}/gamma_hat"][:, k]) <= TOL
        assert rel_l2(g[:, k], g_ref[:, k]) <= TOL
    with pytest.raises(RefMexError) as ei:
        gw.call(node, 2, fix[f"{name}/gamma"])  # adjoint of a gamma-shaped input: wrong rows
    assert ei.value.ident == "combined_quick_gpu:NoValidDoubleMatrix"
    gw.reset()
    gw.lib.ref_clear_mex()


@pytest.mark.gpu
def test_born_mex_rebuilds_for_a_changed_operator_and_a_wider_batch(born_mex):
    b = built("c2")
    gw = born_mex
    g = configs.make_gamma(b.cfg, n_objects=2, seed=3, complex_values=True)
    u1 = gw.call(gw.operator(b.op), 1, g)
    u1b = gw.call(gw.operator(b.op), 1, g)  # same operator, fresh object: the cached plan
    assert np.array_equal(u1, u1b)
    # a different operator of the same sizes: every incident field scaled by 1.5 (1.5 x the output)
    meas = [dataclasses.replace(m, p_incident=1.5 * m.p_incident) for m in b.op.measurements]
    op2 = dataclasses.replace(b.op, measurements=meas)
    u2 = gw.call(gw.operator(op2), 1, g)
    assert rel_l2(u2, 1.5 * u1) <= TOL
    # more objects than the cached plan holds (64): rebuilt wider
    g70 = configs.make_gamma(b.cfg, n_objects=70, seed=4, complex_values=True)
    u3 = gw.call(gw.operator(op2), 1, g70)
    ref = forward_quick_cpu(op2, g70)
    for k in range(70):
        assert rel_l2(u3[:, k], ref[:, k]) <= TOL
    gw.reset()
    gw.lib.ref_clear_mex()


@pytest.mark.gpu
def test_lasso_mex_matches_device_lasso(lasso_mex):
    import torch
    from tests.helpers import make_operator
    b = built("c1")
    gamma_true = configs.make_gamma(b.cfg)
    u = configs.add_noise(forward_quick_cpu(b.op, gamma_true), 25.0, seed=8)
    op = make_operator(b, "lateral", max_objects=1)
    step = 0.9 / op.norm_estimate(8)
    lam = 0.05 * float(np.abs(adjoint_quick_cpu(b.op, u)).max())
    g_dev, _ = op.lasso(torch.from_numpy(u.astype(np.complex64)).cuda(), lam, step, 20)
    node = lasso_mex.operator(b.op)
    d = lasso_mex.dbl
    g_mex = lasso_mex.call_args([node, d(u), d(np.array(lam)), d(np.array(step)), d(np.array(20.0)),
                                 d(np.zeros((b.op.setup.n_points, 1), dtype=complex))])
    assert np.abs(g_mex).max() > 0
    assert rel_l2(g_mex[:, 0], g_dev.cpu().numpy().reshape(-1)) <= 1e-4
    op.close()
    lasso_mex.reset()
    lasso_mex.lib.ref_clear_mex()
