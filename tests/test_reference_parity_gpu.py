"""Device parity against the reference's own outputs.

``tests/golden/reference_gateway.npz`` holds forward and adjoint outputs of the reference's MEX
gateway (``+scattering/combined_quick_gpu.cu``, compiled unchanged and run on the host by
``oracle/ref_mex``; see ``tests/golden/make_reference_golden.py``).  The CUDA paths -- FP32 CUDA
cores, split-BF16 tensor cores over slots and elements, split-BF16 GEMMs against the folded
operator -- must reproduce them within relative L2 <= 1e-5 per column, the operator's bound.
The plans take the reference's own table form (``h_ref`` + ``indices_grid_FOV_shift``).  The
operator tables come from the oracle's builder, whose agreement with the fixture's operator the
CPU suite checks (``tests/test_reference_pinning.py``).
"""

import numpy as np
import pytest

from oracle import configs
from tests.golden.make_reference_golden import CONFIGS, OUT
from tests.helpers import make_operator, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5
FIX = np.load(OUT)


def dev(x):
    return torch.from_numpy(np.asarray(x, dtype=np.complex64)).cuda()


@pytest.mark.parametrize("precision", ["fp32", "bf16x3", "bf16x3-folded"])
@pytest.mark.parametrize("name", CONFIGS)
def test_device_matches_reference_gateway(name, precision):
    if precision == "bf16x3" and name == "c3":
        pytest.skip("3D setups have no element-contraction tensor-core path")
    b = configs.build(configs.small_config(name))
    B = FIX[f"{name}/gamma"].shape[1]
    op = make_operator(b, "reference", max_objects=B)
    op.set_precision(precision)
    for gk, uk in (("gamma", "u"), ("gamma_real", "u_real")):
        u = op.forward(dev(FIX[f"{name}/{gk}"])).cpu().numpy()
        ref = FIX[f"{name}/{uk}"]
        for k in range(ref.shape[1]):
            assert rel_l2(u[:, k], ref[:, k]) <= TOL
    g = op.adjoint(dev(FIX[f"{name}/y"])).cpu().numpy()
    ref = FIX[f"{name}/gamma_hat"]
    for k in range(ref.shape[1]):
        assert rel_l2(g[:, k], ref[:, k]) <= TOL
    assert op.device_status() == 0
    op.close()
