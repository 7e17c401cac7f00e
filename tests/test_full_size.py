"""The benchmark workloads at their full sizes, checked through properties that
hold at any size (the FP64 oracle would take hours there):

- adjointness: <Phi x, y> = <x, Phi^H y> for seeded complex x and y, to 1e-6
  of |Phi x| |y|;
- linearity: Phi(a x1 + b x2) = a Phi x1 + b Phi x2, to relative L2 1e-5.

Every call goes through the C-ABI (ctypes mirror), on the path each workload
benchmarks: split-BF16 tensor cores for the 2D workloads (and FP32 beside
them), FP32 for the 3D matrix array, with its table stored, streamed and generated.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_DOT = 1e-6
TOL_LIN = 1e-5


def _rand(shape, gen):
    re = torch.randn(shape, generator=gen, device="cuda", dtype=torch.float32)
    im = torch.randn(shape, generator=gen, device="cuda", dtype=torch.float32)
    return torch.complex(re, im)


@pytest.mark.parametrize("wname,precision,n_obj,storage", [
    ("2d-batched", "bf16x3", 64, "stored"),
    ("2d-batched", "fp32", 4, "stored"),
    ("2d-gradient", "bf16x3", 1, "stored"),
    ("2d-gradient", "fp32", 1, "stored"),
    ("3d", "fp32", 1, "stored"),
    ("3d", "fp32", 1, "streamed"),
    ("3d", "fp32", 1, "generated"),
])
def test_full_size_adjointness_and_linearity(wname, precision, n_obj, storage):
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload(wname)
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=n_obj, table_storage=storage)
    assert op.table_storage == storage
    op.set_precision(precision)
    gen = torch.Generator(device="cuda").manual_seed(1234)
    x1 = _rand((op.n_points, n_obj), gen)
    x2 = _rand((op.n_points, n_obj), gen)
    y = _rand((op.n_observations, n_obj), gen)
    u1 = op.forward(x1)
    gh = op.adjoint(y)
    lhs = (u1.to(torch.complex128).conj() * y.to(torch.complex128)).sum()
    rhs = (x1.to(torch.complex128).conj() * gh.to(torch.complex128)).sum()
    scale = torch.linalg.vector_norm(u1.to(torch.complex128)) * torch.linalg.vector_norm(y.to(torch.complex128))
    assert float(abs(lhs - rhs) / scale) <= TOL_DOT

    a, b = 0.75 - 0.5j, -1.25 + 0.25j
    u2 = op.forward(x2)
    u12 = op.forward(a * x1 + b * x2)
    ref = a * u1 + b * u2
    rel = torch.linalg.vector_norm(u12 - ref) / torch.linalg.vector_norm(ref)
    assert float(rel) <= TOL_LIN
    assert op.device_status() == 0
    op.close()
