"""Table cache keyed by a hash of the setup (cui_born_plan_create_setup_cached,
cui_born_setup_hash), the counterpart of compute_or_load_hash.m.

CPU tests pin the key: it is deterministic, changes with every field the
device tables depend on, and ignores the receive mixes and the device.  GPU
tests create plans through the cache: the first computes and stores the
table and the incident fields, the next loads them, and both apply
bit-identically; a file written for another setup under the same name is a
hash collision, and a truncated file is rejected.
"""

import copy
import os

import numpy as np
import pytest

from oracle import configs
from tests.helpers import rel_l2, setup_kwargs


def _kw(name="c1"):
    return setup_kwargs(configs.small_config(name))


def test_setup_hash_is_deterministic_and_covers_the_table_inputs():
    from comp_ui_toolbox_gb300.born import setup_hash
    kw = _kw()
    h = setup_hash(**kw)
    assert len(h) == 16 and h == setup_hash(**copy.deepcopy(kw))
    changed = []
    for field, change in [
        ("n_points_axis", lambda k: k.__setitem__("n_points_axis", [k["n_points_axis"][0], k["n_points_axis"][1] + 1])),
        ("delta_axis", lambda k: k.__setitem__("delta_axis", [k["delta_axis"][0], k["delta_axis"][1] * 1.01])),
        ("z_start", lambda k: k.__setitem__("z_start", k["z_start"] + 1e-4)),
        ("width_axis", lambda k: k.__setitem__("width_axis", [k["width_axis"][0] * 0.9])),
        ("absorption", lambda k: k["absorption"].__setitem__("slope_db", k["absorption"]["slope_db"] + 0.1)),
        ("aa_rx_beta", lambda k: k.__setitem__("aa_rx_beta", None)),
        ("f_unique", lambda k: k.__setitem__("f_unique", k["f_unique"] * (1 + 1e-12))),
        ("v_d", lambda k: k["waves"][0].__setitem__("v_d", k["waves"][0]["v_d"] * 1.5)),
    ]:
        k = copy.deepcopy(kw)
        change(k)
        changed.append((field, setup_hash(**k) != h))
    assert all(c for _, c in changed), changed
    k = copy.deepcopy(kw)  # receive mixes and device do not enter the tables
    for w in k["waves"]:
        for m in w["mixes"]:
            m["response"] = m["response"] * 2.0
    assert setup_hash(**k, device=3) == h


@pytest.mark.gpu
def test_cache_stores_then_loads_bit_identical_tables(tmp_path):
    torch = pytest.importorskip("torch")
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.born import setup_hash
    b = configs.build(configs.small_config("c2"))
    kw = setup_kwargs(b.cfg)
    B = b.cfg.n_objects
    first = OperatorBorn.from_setup(**kw, max_objects=B, cache_dir=str(tmp_path))
    assert first.loaded_from_cache == 0
    path = tmp_path / f"cui_born_{setup_hash(**kw)}.tables"
    assert path.exists() and os.path.getsize(path) >= first.info["table_bytes"] + first.info["incident_bytes"]
    assert not list(tmp_path.glob("*.tmp"))
    second = OperatorBorn.from_setup(**kw, max_objects=B, cache_dir=str(tmp_path))
    assert second.loaded_from_cache == 1
    plain = OperatorBorn.from_setup(**kw, max_objects=B)
    g = torch.from_numpy(configs.make_gamma(b.cfg, seed=5).astype(np.complex64)).cuda()
    u1, u2, u0 = first.forward(g), second.forward(g), plain.forward(g)
    a1, a2 = first.adjoint(u0), second.adjoint(u0)
    torch.cuda.synchronize()
    assert torch.equal(u1, u2) and torch.equal(u1, u0) and torch.equal(a1, a2)
    # other receive mixes, same tables: loaded, and equal to an uncached plan of that setup
    k2 = copy.deepcopy(kw)
    for w in k2["waves"]:
        for m in w["mixes"]:
            m["response"] = m["response"] * (0.5 - 0.25j)
    third = OperatorBorn.from_setup(**k2, max_objects=B, cache_dir=str(tmp_path))
    assert third.loaded_from_cache == 1
    ref = OperatorBorn.from_setup(**k2, max_objects=B)
    assert torch.equal(third.forward(g), ref.forward(g))
    assert rel_l2(third.forward(g).cpu().numpy(), (u0 * (0.5 - 0.25j)).cpu().numpy()) <= 1e-6


@pytest.mark.gpu
def test_cache_rejects_collisions_and_truncated_files(tmp_path):
    pytest.importorskip("torch")
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.born import CuiError, setup_hash
    kw_a, kw_b = _kw("c1"), _kw("c2")
    OperatorBorn.from_setup(**kw_a, cache_dir=str(tmp_path))
    OperatorBorn.from_setup(**kw_b, cache_dir=str(tmp_path))
    pa = tmp_path / f"cui_born_{setup_hash(**kw_a)}.tables"
    pb = tmp_path / f"cui_born_{setup_hash(**kw_b)}.tables"
    data_b = pb.read_bytes()
    pb.write_bytes(pa.read_bytes())  # a file of setup a under setup b's name
    with pytest.raises(CuiError, match="hash collision"):
        OperatorBorn.from_setup(**kw_b, cache_dir=str(tmp_path))
    pb.write_bytes(data_b[: len(data_b) - 100])
    with pytest.raises(CuiError, match="truncated"):
        OperatorBorn.from_setup(**kw_b, cache_dir=str(tmp_path))
