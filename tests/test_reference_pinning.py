"""The oracle pinned to the reference's own code (no GPU).

``tests/golden/reference_gateway.npz`` holds outputs of the reference's MEX gateway
``+scattering/combined_quick_gpu.cu`` (compiled unchanged, run on the host by ``oracle/ref_mex``;
generated by ``tests/golden/make_reference_golden.py``).  The gateway computes in FP32, so the
FP64 oracle must agree with it to FP32 rounding: relative L2 <= 1e-6 per column, for complex and
real (promoted, ``combined_quick_gpu.cu:424-437``) gamma and for the adjoint.  Where the runner
library has been built (a machine with the reference checkout), the live gateway is also checked:
more seeds, every small configuration, an all-zero gamma (no occupied points: zero output,
``:496``) and its argument errors.
"""

import numpy as np
import pytest

from oracle import adjoint_quick_cpu, configs, forward_quick_cpu
from oracle import ref_runner
from tests.golden.make_reference_golden import CONFIGS, OUT, table_checksums
from tests.helpers import rel_l2

TOL_REF = 1e-6
FIX = np.load(OUT)
_BUILT = {}


def built(name):
    if name not in _BUILT:
        _BUILT[name] = configs.build(configs.small_config(name))
    return _BUILT[name]


def columns(a, b, tol):
    for k in range(b.shape[1]):
        assert rel_l2(a[:, k], b[:, k]) <= tol, k


@pytest.mark.parametrize("name", CONFIGS)
def test_oracle_builds_the_fixture_operator(name):
    np.testing.assert_allclose(table_checksums(built(name)), FIX[f"{name}/checksums"], rtol=1e-12)


@pytest.mark.parametrize("name", CONFIGS)
def test_oracle_matches_reference_gateway(name):
    b = built(name)
    columns(forward_quick_cpu(b.op, FIX[f"{name}/gamma"]), FIX[f"{name}/u"], TOL_REF)
    columns(forward_quick_cpu(b.op, FIX[f"{name}/gamma_real"]), FIX[f"{name}/u_real"], TOL_REF)
    columns(adjoint_quick_cpu(b.op, FIX[f"{name}/y"]), FIX[f"{name}/gamma_hat"], TOL_REF)


def test_fixture_shapes_follow_the_gateway_layout():
    for name in CONFIGS:
        b = built(name)
        assert FIX[f"{name}/u"].shape == (b.op.n_observations, FIX[f"{name}/gamma"].shape[1])
        assert FIX[f"{name}/gamma_hat"].shape == (b.op.setup.n_points, FIX[f"{name}/y"].shape[1])


live = pytest.mark.skipif(not ref_runner.available(), reason="reference runner not built (needs the reference checkout)")


@live
@pytest.mark.parametrize("name", CONFIGS)
def test_live_gateway_matches_oracle(name):
    b = built(name)
    gw = ref_runner.ReferenceGateway()
    node = gw.operator(b.op)
    rng = np.random.default_rng(17)
    g = configs.make_gamma(b.cfg, n_objects=3, seed=71, complex_values=True)
    columns(gw.call(node, 1, g), forward_quick_cpu(b.op, g), TOL_REF)
    y = rng.standard_normal((b.op.n_observations, 2)) + 1j * rng.standard_normal((b.op.n_observations, 2))
    columns(gw.call(node, 2, y), adjoint_quick_cpu(b.op, y), TOL_REF)
    zero = gw.call(node, 1, np.zeros((b.op.setup.n_points, 2)))
    assert zero.shape == (b.op.n_observations, 2) and not np.any(zero)
    gw.reset()


@live
def test_live_gateway_argument_errors():
    b = built("c1")
    gw = ref_runner.ReferenceGateway()
    node = gw.operator(b.op)
    g = configs.make_gamma(b.cfg)
    cases = [((1, np.zeros((3, 1))), "combined_quick_gpu:NoValidDoubleMatrix"),
             ((np.array([1.0, 2.0]), g), "combined_quick_gpu:NoNumericScalarMode"),
             ((1j, g), "combined_quick_gpu:NoNumericScalarMode")]
    for args, ident in cases:
        with pytest.raises(ref_runner.RefMexError) as ei:
            gw.call(node, *args)
        assert ei.value.ident == ident
    with pytest.raises(ref_runner.RefMexError) as ei:
        gw.call(gw.operator(b.op, setup_class="scattering.sequences.setups.setup"), 1, g)
    assert ei.value.ident == "combined_quick_gpu:NoSymmetricGridsSetup"
    with pytest.raises(ref_runner.RefMexError) as ei:
        gw.call(gw.operator(b.op, gpu_class="scattering.options.gpu_off"), 1, g)
    assert ei.value.ident == "combined_quick_gpu:NoScatteringOptionsGPUActive"
    with pytest.raises(ref_runner.RefMexError) as ei:
        gw.call(node, 1, g, nrhs=2)
    assert ei.value.ident == "combined_quick_gpu:NumberArguments"
    gw.reset()
