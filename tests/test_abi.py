"""CPU checks of the C-ABI library: it builds, loads and exports every symbol
``include/cui_born.h`` declares; argument validation answers without a GPU.
No compute call is made here."""

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "cui_born.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cui_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from comp_ui_toolbox_gb300 import build
    build.build()
    from comp_ui_toolbox_gb300.born import load_library
    return load_library()


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ["cui_born_plan_create", "cui_born_plan_destroy", "cui_born_forward", "cui_born_adjoint",
              "cui_born_vjp", "cui_born_combined_host", "cui_born_size", "cui_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_mirror_binds_every_symbol():
    from comp_ui_toolbox_gb300.born import _SIGNATURES
    assert set(_SIGNATURES) == set(declared_functions())


def test_status_strings_and_null_arguments(lib):
    assert lib.cui_status_string(0) == b"CUI_OK"
    assert lib.cui_status_string(2) == b"CUI_ERR_UNSUPPORTED_SETUP"
    assert lib.cui_born_plan_destroy(None) == 0
    n = C.c_int64()
    assert lib.cui_born_size(None, C.byref(n), None) == 1
    assert lib.cui_born_forward(None, None, 0, 1, None, 0, None) == 1
    assert b"plan" in lib.cui_last_error()
    out = C.c_void_p()
    assert lib.cui_born_plan_create(None, 1, C.byref(out)) == 1
    assert out.value is None


def test_descriptor_validation_before_any_device_call(lib):
    from comp_ui_toolbox_gb300.born import BornDesc
    d = BornDesc()
    d.n_dims = 4
    out = C.c_void_p()
    assert lib.cui_born_plan_create(C.byref(d), 1, C.byref(out)) == 1
    assert b"n_dims" in lib.cui_last_error()
    d.n_dims = 2
    d.n_points_axis[0] = 8
    d.n_points_axis[1] = 4
    d.n_elements_axis[0] = 2
    d.n_points_per_pitch[0] = 2
    d.n_f_unique = 1
    d.n_measurements = 0
    assert lib.cui_born_plan_create(C.byref(d), 1, C.byref(out)) == 1
    assert b"measurement" in lib.cui_last_error()


def test_launch_counter_starts_readable(lib):
    assert lib.cui_launch_count() >= 0


def test_c_harness_builds_against_the_header(lib):
    """The plain C driver compiles as C99 against include/cui_born.h and links the library."""
    from comp_ui_toolbox_gb300 import build
    assert build.build_harness().exists()


def test_table_storage_names_match_the_header_and_null_arguments(lib):
    """The Python names of cui_table_storage carry the header's values; the storage query and the
    launch-shape entry points reject NULL plans without a device call."""
    from comp_ui_toolbox_gb300.born import _TABLE_STORAGE
    text = HEADER.read_text()
    values = {m.group(1): int(m.group(2)) for m in re.finditer(r"CUI_STORAGE_([A-Z]+)\s*=\s*(\d+)", text)}
    assert {k.upper(): v for k, v in _TABLE_STORAGE.items()} == values
    s = C.c_int32()
    assert lib.cui_born_plan_table_storage(None, C.byref(s)) == 1
    assert lib.cui_born_set_launch_shapes(None, 0, 0, 0) == 1
    assert lib.cui_born_autotune_config(None, None, None, None) == 1
    out = C.c_void_p()
    assert lib.cui_born_plan_create_setup_ex(None, 1, 0, None, C.byref(out), None) == 1
    assert out.value is None


def test_unknown_table_storage_is_rejected_on_the_host():
    from comp_ui_toolbox_gb300 import OperatorBorn
    from oracle import configs
    from tests.helpers import setup_kwargs
    with pytest.raises(KeyError):
        OperatorBorn.from_setup(**setup_kwargs(configs.small_config("c3")), table_storage="compressed")


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """Every struct the Python mirror passes through the C-ABI has the header's size and field
    offsets (a C program compiled against include/cui_born.h prints them)."""
    import json
    import shutil
    import subprocess
    from comp_ui_toolbox_gb300 import born
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"cui_mix_desc": born.MixDesc, "cui_measurement_desc": born.MeasurementDesc,
             "cui_born_desc": born.BornDesc, "cui_absorption_desc": born.AbsorptionDesc,
             "cui_wave_desc": born.WaveDesc, "cui_born_setup_desc": born.SetupDesc,
             "cui_born_timing": born.BornTiming, "cui_born_info": born.BornInfo}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "cui_born.h"', "int main(void) {",
             'printf("{");']
    first = True
    for cname, py in pairs.items():
        for fname, _ in py._fields_:
            sep = "" if first else ","
            first = False
            lines.append(f'printf("{sep}\\"{cname}.{fname}\\": %zu", offsetof({cname}, {fname}));')
        lines.append(f'printf(",\\"{cname}\\": %zu", sizeof({cname}));')
    lines += ['printf("}\\n");', "return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", f"-I{HEADER.parent}", str(src), "-o", str(exe)], check=True)
    got = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    for cname, py in pairs.items():
        assert got[cname] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[f"{cname}.{fname}"] == getattr(py, fname).offset, f"{cname}.{fname}"
