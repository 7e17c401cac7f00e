"""Python host mirror of the reference's Born-operator interface.

Mirrors the calls a user of ``scattering.operator_born`` makes
(``+scattering/operator_born.m``, ``+scattering/operator.m``):

* ``OperatorBorn.forward(gamma)``   -> ``forward_scalar`` / ``op * gamma``   (``operator_born.m:37-44``, ``:174-238``)
* ``OperatorBorn.adjoint(u)``       -> ``adjoint_scalar``                    (``operator_born.m:243-320``)
* ``OperatorBorn.combined_scalar(mode, x)`` -> ``operator.combined_scalar``  (``operator.m:1019-1072``; mode 0 size,
  1 forward, 2 adjoint)
* ``OperatorBorn.vjp(gamma, u)``    -> gradient of ``0.5*||Phi gamma - u||^2`` used by the solvers
  (``operator.m:717``)

All arithmetic runs in ``libcui_born.so`` through its C-ABI (``include/cui_born.h``).
NumPy inputs take the FP64 host path (``cui_born_combined_host``, the MEX
semantics); CUDA ``torch`` tensors take the FP32 device path.  There is no CPU
fallback: without the compiled library every entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

__all__ = ["OperatorBorn", "CuiError", "load_library", "BornForward", "born_forward", "launch_count"]

_LIB_PATH = Path(__file__).resolve().parent / "libcui_born.so"

STATUS = {0: "CUI_OK", 1: "CUI_ERR_INVALID_ARG", 2: "CUI_ERR_UNSUPPORTED_SETUP", 3: "CUI_ERR_OOM",
          4: "CUI_ERR_CUDA", 5: "CUI_ERR_TIMEOUT", 6: "CUI_ERR_NUMERIC", 7: "CUI_ERR_NO_DEVICE"}

# reference MEX error identifiers for each status (+scattering/combined_quick_gpu.cu:201-428, .h:43)
MEX_ID = {1: "combined_quick_gpu:NoValidDoubleMatrix", 2: "combined_quick_gpu:NoSymmetricGridsSetup",
          3: "adjoint_quick_gpu:ErrorCUDA", 4: "adjoint_quick_gpu:ErrorCUDA", 5: "adjoint_quick_gpu:ErrorCUDA",
          6: "combined_quick_gpu:NoComplexDoubles", 7: "combined_quick_gpu:NoCUDADevices"}


class CuiError(RuntimeError):
    """A libcui_born call failed; ``status`` is the cui_status code."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.identifier = MEX_ID.get(status, "combined_quick_gpu:Error")
        super().__init__(f"{STATUS.get(status, status)}: {message} [{self.identifier}]")


class c64(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class MixDesc(C.Structure):
    _fields_ = [("n_f", C.c_int32), ("indices_f_to_unique", C.POINTER(C.c_int32)),
                ("n_active", C.c_int32), ("indices_active", C.POINTER(C.c_int32)),
                ("prefactors", C.c_void_p)]


class MeasurementDesc(C.Structure):
    _fields_ = [("n_f", C.c_int32), ("indices_f_to_unique", C.POINTER(C.c_int32)),
                ("p_incident", C.c_void_p), ("n_mixes", C.c_int32), ("mixes", C.POINTER(MixDesc))]


class BornDesc(C.Structure):
    _fields_ = [("n_dims", C.c_int32), ("n_points_axis", C.c_int32 * 3), ("n_elements_axis", C.c_int32 * 2),
                ("n_points_per_pitch", C.c_int32 * 2), ("n_f_unique", C.c_int32), ("table_form", C.c_int32),
                ("h_ref", C.c_void_p), ("indices_grid_FOV_shift", C.POINTER(C.c_int32)),
                ("h_lateral", C.c_void_p), ("n_measurements", C.c_int32),
                ("measurements", C.POINTER(MeasurementDesc)), ("device", C.c_int32)]


class AbsorptionDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("c", C.c_double), ("constant_db", C.c_double), ("slope_db", C.c_double),
                ("exponent", C.c_double), ("f_ref", C.c_double), ("dispersion", C.c_int32)]


class WaveDesc(C.Structure):
    _fields_ = [("n_f", C.c_int32), ("indices_f_to_unique", C.POINTER(C.c_int32)), ("v_d", C.c_void_p),
                ("n_mixes", C.c_int32), ("mixes", C.POINTER(MixDesc))]


class SetupDesc(C.Structure):
    _fields_ = [("n_dims", C.c_int32), ("n_points_axis", C.c_int32 * 3), ("delta_axis", C.c_double * 3),
                ("z_start", C.c_double), ("n_elements_axis", C.c_int32 * 2), ("pitch_axis", C.c_double * 2),
                ("width_axis", C.c_double * 2), ("n_face_axis", C.c_int32 * 2), ("absorption", AbsorptionDesc),
                ("aa_tx_beta", C.c_double), ("aa_rx_beta", C.c_double), ("n_f_unique", C.c_int32),
                ("f_unique", C.POINTER(C.c_double)), ("n_measurements", C.c_int32),
                ("waves", C.POINTER(WaveDesc)), ("device", C.c_int32),
                ("face_apodization", C.POINTER(C.c_double)), ("lens_focus_axis", C.c_double * 2),
                ("lens_c", C.c_double)]


class BornTiming(C.Structure):
    _fields_ = [("n_forward", C.c_int64), ("n_adjoint", C.c_int64), ("ms_forward", C.c_double),
                ("ms_adjoint", C.c_double)]


class BornInfo(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("n_points", "n_observations", "n_elements", "n_slots", "n_f_unique",
                                         "table_bytes", "incident_bytes", "workspace_bytes", "contraction_macs",
                                         "channel_macs", "folded_bytes", "folded_sums", "device_allocations")]


_lib = None

# cui_table_storage
_TABLE_STORAGE = {"auto": 0, "stored": 1, "generated": 2, "streamed": 3}

# every symbol include/cui_born.h declares, with its ctypes signature
_SIGNATURES = {
    "cui_born_plan_create": (C.c_int, [C.POINTER(BornDesc), C.c_int32, C.POINTER(C.c_void_p)]),
    "cui_born_plan_create_setup": (C.c_int, [C.POINTER(SetupDesc), C.c_int32, C.POINTER(C.c_void_p)]),
    "cui_born_plan_create_setup_cached": (C.c_int, [C.POINTER(SetupDesc), C.c_int32, C.c_char_p,
                                                    C.POINTER(C.c_void_p), C.POINTER(C.c_int32)]),
    "cui_born_setup_hash": (C.c_int, [C.POINTER(SetupDesc), C.c_char_p]),
    "cui_born_plan_create_setup_ex": (C.c_int, [C.POINTER(SetupDesc), C.c_int32, C.c_int32, C.c_char_p,
                                                C.POINTER(C.c_void_p), C.POINTER(C.c_int32)]),
    "cui_born_plan_table_storage": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "cui_born_autotune_config": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                           C.POINTER(C.c_int32)]),
    "cui_born_set_launch_shapes": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "cui_born_plan_destroy": (C.c_int, [C.c_void_p]),
    "cui_born_plan_info": (C.c_int, [C.c_void_p, C.POINTER(BornInfo)]),
    "cui_born_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "cui_born_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]),
    "cui_born_forward_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                                          C.c_void_p]),
    "cui_born_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]),
    "cui_born_vjp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                               C.c_int64, C.c_void_p, C.c_void_p]),
    "cui_born_lasso": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p,
                                 C.c_float, C.c_int32, C.c_void_p, C.c_void_p]),
    "cui_born_combined_host": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                                         C.c_int64]),
    "cui_born_vjp_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32,
                                    C.c_void_p, C.c_int64, C.POINTER(C.c_double)]),
    "cui_born_set_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "cui_born_host_path": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "cui_born_lasso_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                                      C.c_void_p, C.c_float, C.c_int32]),
    "cui_born_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int64]),
    "cui_born_set_occupancy_limit": (C.c_int, [C.c_void_p, C.c_int64]),
    "cui_born_energy_rx": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "cui_born_omp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.POINTER(C.c_int64), C.c_void_p,
                               C.POINTER(C.c_float), C.POINTER(C.c_int32), C.c_void_p]),
    "cui_born_cosamp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.POINTER(C.c_int64),
                                  C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int32), C.c_void_p]),
    "cui_born_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_void_p]),
    "cui_born_plan_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "cui_born_timing_enable": (C.c_int, [C.c_void_p, C.c_int32]),
    "cui_born_timing_read": (C.c_int, [C.c_void_p, C.POINTER(BornTiming)]),
    "cui_status_string": (C.c_char_p, [C.c_int]),
    "cui_last_error": (C.c_char_p, []),
    "cui_launch_count": (C.c_int64, []),
}


def load_library(path: Optional[os.PathLike] = None) -> C.CDLL:
    """Load libcui_born.so (built in-tree by ``comp_ui_toolbox_gb300/build.py``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else _LIB_PATH
    if not p.exists():
        raise CuiError(4, f"{p} is missing: build it with `python -m comp_ui_toolbox_gb300.build` "
                          "(the operator has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def launch_count() -> int:
    """Kernel launches issued by the library in this process."""
    return int(load_library().cui_launch_count())


def _check(status: int):
    if status != 0:
        msg = load_library().cui_last_error().decode(errors="replace")
        raise CuiError(status, msg)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _c128_f(a) -> np.ndarray:
    """Complex FP64 array in column-major (MATLAB) order."""
    return np.asfortranarray(np.asarray(a, dtype=np.complex128))


def _get(obj, key):
    return obj[key] if isinstance(obj, dict) else getattr(obj, key)


def _mix_array(mixes_in, weight_key, keep):
    """ctypes array of cui_mix_desc; ``weight_key`` names the prefactor / response field."""
    mixes = (MixDesc * max(1, len(mixes_in)))()
    keep.append(mixes)
    for k, mx in enumerate(mixes_in):
        mf = _i32(np.asarray(_get(mx, "f_idx")) + 1)
        act = _i32(np.asarray(_get(mx, "active")) + 1)
        wts = _c128_f(_get(mx, weight_key))
        keep += [mf, act, wts]
        mixes[k].n_f = len(mf)
        mixes[k].indices_f_to_unique = mf.ctypes.data_as(C.POINTER(C.c_int32))
        mixes[k].n_active = len(act)
        mixes[k].indices_active = act.ctypes.data_as(C.POINTER(C.c_int32))
        mixes[k].prefactors = wts.ctypes.data
    return mixes


class OperatorBorn:
    """Persistent GB300 Born operator built from the reference operator's tables.

    Parameters mirror what ``combined_quick_gpu`` reads from
    ``operator_born`` (``combined_quick_gpu.cu:203-393``):

    * ``n_points_axis``: FOV grid points, lateral axes then axial;
    * ``n_elements_axis`` / ``n_points_per_pitch``: array elements and grid
      points per pitch along each lateral axis;
    * ``h_lateral``: lateral-offset table ``(F, Nz, [No_y,] No_x)``, or
      ``h_ref`` ``(F, P)`` with ``indices_grid_FOV_shift`` ``(P, E)``
      (1-based) -- the reference's own symmetric-grid representation;
    * ``measurements``: sequence of objects or dicts with ``f_idx`` (0-based
      global frequency indices), ``p_incident`` ``(F_w, P)`` and ``mixes``,
      each with ``f_idx`` (0-based into the measurement's frequencies),
      ``active`` (0-based element indices) and ``pref`` ``(F_mix, n_active)``.
    """

    def __init__(self, *, n_points_axis: Sequence[int], n_elements_axis: Sequence[int],
                 n_points_per_pitch: Sequence[int], n_f_unique: int, measurements,
                 h_lateral: Optional[np.ndarray] = None, h_ref: Optional[np.ndarray] = None,
                 indices_grid_FOV_shift: Optional[np.ndarray] = None, device: int = 0, max_objects: int = 1):
        lib = load_library()
        self._lib = lib
        self._plan = C.c_void_p()
        keep = []  # host arrays must outlive plan creation only
        n_dims = len(n_points_axis)
        d = BornDesc()
        d.n_dims = n_dims
        for k, v in enumerate(n_points_axis):
            d.n_points_axis[k] = int(v)
        for k, v in enumerate(n_elements_axis):
            d.n_elements_axis[k] = int(v)
        for k, v in enumerate(n_points_per_pitch):
            d.n_points_per_pitch[k] = int(v)
        d.n_f_unique = int(n_f_unique)
        if h_lateral is not None:
            t = np.ascontiguousarray(np.asarray(h_lateral, dtype=np.complex128))
            keep.append(t)
            d.table_form = 1
            d.h_lateral = t.ctypes.data
        else:
            if h_ref is None or indices_grid_FOV_shift is None:
                raise ValueError("give h_lateral, or h_ref together with indices_grid_FOV_shift")
            h = _c128_f(h_ref)
            m = np.asfortranarray(np.asarray(indices_grid_FOV_shift, dtype=np.int32))
            keep += [h, m]
            d.table_form = 0
            d.h_ref = h.ctypes.data
            d.indices_grid_FOV_shift = m.ctypes.data_as(C.POINTER(C.c_int32))
        meas = (MeasurementDesc * len(measurements))()
        for w, ms in enumerate(measurements):
            f_idx = _i32(np.asarray(_get(ms, "f_idx")) + 1)
            p_in = _c128_f(_get(ms, "p_incident"))
            mixes_in = list(_get(ms, "mixes"))
            keep += [f_idx, p_in]
            meas[w].n_f = len(f_idx)
            meas[w].indices_f_to_unique = f_idx.ctypes.data_as(C.POINTER(C.c_int32))
            meas[w].p_incident = p_in.ctypes.data
            meas[w].n_mixes = len(mixes_in)
            meas[w].mixes = _mix_array(mixes_in, "pref", keep)
        d.n_measurements = len(measurements)
        d.measurements = meas
        d.device = int(device)
        _check(lib.cui_born_plan_create(C.byref(d), int(max_objects), C.byref(self._plan)))
        self._finish(max_objects, device)

    @classmethod
    def from_setup(cls, *, device: int = 0, max_objects: int = 1, cache_dir: Optional[str] = None,
                   table_storage: str = "auto", **setup) -> "OperatorBorn":
        """Plan whose tables the GPU computes from the discretised setup (``setup_desc`` lists
        the keyword arguments).

        With ``cache_dir`` the plan goes through the table cache
        (``cui_born_plan_create_setup_cached``, ``compute_or_load_hash.m``): the table and the
        incident fields are loaded from ``cache_dir/cui_born_<setup hash>.tables`` when that
        file exists, else computed and stored there.  ``loaded_from_cache`` is then 1 (loaded),
        0 (computed and stored) or -1 (computed; storing failed).

        ``table_storage`` (``cui_born_plan_create_setup_ex``): ``"stored"`` builds the lateral
        table once; ``"streamed"`` (3D setups) regenerates it every apply one chunk of
        frequencies at a time into a chunk buffer; ``"generated"`` (3D) never stores any of it,
        the kernels compute each entry where they use it; ``"auto"`` stores it unless it does
        not fit in device memory.  ``self.table_storage`` says which the plan uses.
        """
        self = cls.__new__(cls)
        lib = load_library()
        self._lib = lib
        self._plan = C.c_void_p()
        d, keep = setup_desc(device=device, **setup)
        self.loaded_from_cache = None
        storage = _TABLE_STORAGE[table_storage]
        if cache_dir is None and storage == 0:
            _check(lib.cui_born_plan_create_setup(C.byref(d), int(max_objects), C.byref(self._plan)))
        else:
            loaded = C.c_int32(0)
            _check(lib.cui_born_plan_create_setup_ex(C.byref(d), int(max_objects), storage,
                                                     None if cache_dir is None else str(cache_dir).encode(),
                                                     C.byref(self._plan), C.byref(loaded)))
            if cache_dir is not None:
                self.loaded_from_cache = loaded.value
        del keep
        self._finish(max_objects, device)
        mode = C.c_int32(0)
        _check(lib.cui_born_plan_table_storage(self._plan, C.byref(mode)))
        self.table_storage = {v: k for k, v in _TABLE_STORAGE.items()}[mode.value]
        return self

    def _finish(self, max_objects, device):
        lib = self._lib
        self.max_objects = int(max_objects)
        info = BornInfo()
        _check(lib.cui_born_plan_info(self._plan, C.byref(info)))
        self.info = {n: int(getattr(info, n)) for n, _ in BornInfo._fields_}
        self.n_observations = self.info["n_observations"]
        self.n_points = self.info["n_points"]
        self.device = int(device)
        self.table_storage = "stored"
        self.precision = "fp32"  # the path a new plan runs (cui_born_set_precision changes it)

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "_plan", None) and self._plan.value:
            self._lib.cui_born_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    PRECISIONS = {"fp32": 0, "bf16x3": 1, "bf16x3-folded": 2}

    def set_precision(self, precision: str) -> None:
        """``"fp32"`` (CUDA cores), ``"bf16x3"`` (split-BF16 tcgen05 tensor cores over slots and
        elements) or ``"bf16x3-folded"`` (split-BF16 tcgen05 GEMMs against the operator folded over
        its receive mixes and stored in device memory, built on the first switch)."""
        _check(self._lib.cui_born_set_precision(self._plan, self.PRECISIONS[precision]))
        self.precision = precision

    def autotune(self, n_objects: int = 1) -> dict:
        """Keep the faster of the FP32 and split-BF16 paths for ``n_objects`` columns and, on the
        split-BF16 path, the fastest launch shapes (``cui_born_autotune``); returns the choice,
        both times and the launch shapes (``cui_born_autotune_config``)."""
        import torch
        choice = C.c_int32(0)
        ms = (C.c_double * 2)()
        st = torch.cuda.current_stream().cuda_stream
        _check(self._lib.cui_born_autotune(self._plan, int(n_objects), C.byref(choice), ms, st))
        tiles, fwd, adj = C.c_int32(0), C.c_int32(0), C.c_int32(0)
        _check(self._lib.cui_born_autotune_config(self._plan, C.byref(tiles), C.byref(fwd), C.byref(adj)))
        self.precision = "bf16x3" if choice.value == 1 else "fp32"  # the plan now runs the kept path
        return {"precision": self.precision, "ms_fp32": ms[0], "ms_bf16x3": ms[1],
                "launch_shapes": {"narrow_tiles": tiles.value, "fwd_blocks": fwd.value or "rule",
                                  "adj_blocks": adj.value or "rule"}}

    def set_launch_shapes(self, narrow_tiles: int = 0, fwd_blocks: int = 0, adj_blocks: int = 0) -> None:
        """Launch shapes of the split-BF16 line-unit kernels (``cui_born_set_launch_shapes``; 0: the rule)."""
        _check(self._lib.cui_born_set_launch_shapes(self._plan, int(narrow_tiles), int(fwd_blocks), int(adj_blocks)))

    def refresh_info(self) -> dict:
        """Re-read the plan's work and storage figures (``cui_born_plan_info``), for instance after
        switching to the folded operator, which adds its matrix."""
        info = BornInfo()
        _check(self._lib.cui_born_plan_info(self._plan, C.byref(info)))
        self.info = {n: int(getattr(info, n)) for n, _ in BornInfo._fields_}
        return self.info

    def host_path(self) -> str:
        """``"direct"`` when the host entry points' kernels read and write the caller's arrays through
        the host page tables, ``"staging"`` when the data pass through pinned buffers."""
        d = C.c_int32()
        _check(self._lib.cui_born_host_path(self._plan, C.byref(d)))
        return "direct" if d.value else "staging"

    def set_wait_limit(self, nanoseconds: int = 0) -> None:
        """Wall-clock limit of the tensor-core kernels' waits (``cui_born_set_wait_limit``; 0: 1 s)."""
        _check(self._lib.cui_born_set_wait_limit(self._plan, int(nanoseconds)))

    def set_occupancy_limit(self, max_points: int = -1) -> None:
        """FP32 forward: contract over the occupied points when there are at most ``max_points``
        (``cui_born_set_occupancy_limit``; -1: N_points / 16 with a stored table, / 32 with a
        streamed or generated one; 0: always dense)."""
        _check(self._lib.cui_born_set_occupancy_limit(self._plan, int(max_points)))

    def device_status(self) -> int:
        """Read and clear the device status word (raises CuiError on a timed-out wait)."""
        s = C.c_int32()
        _check(self._lib.cui_born_plan_status(self._plan, C.byref(s)))
        return s.value

    def timing(self, enable: Optional[bool] = None) -> dict:
        """Enable/disable per-kernel event timing, or read (and clear) the sums."""
        if enable is not None:
            _check(self._lib.cui_born_timing_enable(self._plan, int(bool(enable))))
            return {}
        t = BornTiming()
        _check(self._lib.cui_born_timing_read(self._plan, C.byref(t)))
        return {n: getattr(t, n) for n, _ in BornTiming._fields_}

    @property
    def size(self):
        """Operator size ``(N_observations, N_points)`` (``operator.m:1042-1045``)."""
        return self.n_observations, self.n_points

    # ------------------------------------------------------------------ host (FP64)
    def _host_apply(self, mode: int, x: np.ndarray) -> np.ndarray:
        x = np.asarray(x)
        vec = x.ndim == 1
        x2 = _c128_f(x[:, None] if vec else x)
        rows_out = self.n_observations if mode == 1 else self.n_points
        out = np.zeros((rows_out, x2.shape[1]), dtype=np.complex128, order="F")
        _check(self._lib.cui_born_combined_host(self._plan, mode, x2.ctypes.data, x2.shape[0], x2.shape[1],
                                                out.ctypes.data, rows_out))
        return out[:, 0] if vec else out

    # ------------------------------------------------------------------ device (FP32)
    @staticmethod
    def _cols(t):
        """(rows, B) column-major view of a CUDA complex64 tensor as a (B, rows) contiguous tensor."""
        import torch
        if t.dtype != torch.complex64 or not t.is_cuda:
            raise TypeError("device applies take CUDA complex64 tensors")
        vec = t.dim() == 1
        tt = t[:, None] if vec else t
        return tt.t().contiguous(), vec

    def _dev_apply(self, mode: int, x):
        import torch
        xc, vec = self._cols(x)
        B, rows_in = xc.shape
        rows_out = self.n_observations if mode == 1 else self.n_points
        out = torch.empty((B, rows_out), dtype=torch.complex64, device=x.device)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        fn = self._lib.cui_born_forward if mode == 1 else self._lib.cui_born_adjoint
        _check(fn(self._plan, xc.data_ptr(), rows_in, B, out.data_ptr(), rows_out, stream))
        out = out.t()
        return out[:, 0] if vec else out

    def _is_torch(self, x):
        try:
            import torch
        except ImportError:
            return False
        return isinstance(x, torch.Tensor)

    def forward(self, gamma):
        """``u = Phi * gamma`` (``operator_born.m:37-44``)."""
        return self._dev_apply(1, gamma) if self._is_torch(gamma) else self._host_apply(1, gamma)

    def adjoint(self, u):
        """``gamma_hat = Phi^H * u`` (``operator_born.m:243-320``)."""
        return self._dev_apply(2, u) if self._is_torch(u) else self._host_apply(2, u)

    __mul__ = forward

    def combined_scalar(self, mode: int, x=None):
        """``operator.combined_scalar`` (``operator.m:1019-1072``): 0 size, 1 forward, 2 adjoint."""
        if mode == 0:
            return self.size
        if mode == 1:
            return self.forward(x)
        if mode == 2:
            return self.adjoint(x)
        raise CuiError(1, "mode must be 0, 1 or 2")

    def vjp(self, gamma, u_meas, out=None):
        """Gradient and value of ``0.5*||Phi gamma - u||^2`` per column: ``(grad, loss)``.

        Host (numpy) inputs follow the MEX semantics; column-major complex128
        arrays (MATLAB's layout) pass through without a copy, and ``out`` (a
        column-major complex128 array of gamma's shape) receives the gradient
        without a new allocation.
        """
        if self._is_torch(gamma):
            import torch
            gc, vec = self._cols(gamma)
            uc, _ = self._cols(u_meas)
            B = gc.shape[0]
            grad = torch.empty_like(gc)
            loss = torch.empty(B, dtype=torch.float32, device=gamma.device)
            stream = torch.cuda.current_stream(gamma.device).cuda_stream
            _check(self._lib.cui_born_vjp(self._plan, gc.data_ptr(), self.n_points, uc.data_ptr(),
                                          self.n_observations, B, grad.data_ptr(), self.n_points,
                                          loss.data_ptr(), stream))
            grad = grad.t()
            return (grad[:, 0], loss[0]) if vec else (grad, loss)
        g = np.asarray(gamma)
        vec = g.ndim == 1
        g2 = _c128_f(g[:, None] if vec else g)
        u2 = _c128_f(np.asarray(u_meas)[:, None] if vec else u_meas)
        B = g2.shape[1]
        if out is not None:
            grad = out[:, None] if out.ndim == 1 else out
            if grad.dtype != np.complex128 or not grad.flags.f_contiguous or grad.shape != (self.n_points, B):
                raise CuiError(1, "out must be a column-major complex128 array of gamma's shape")
        else:
            grad = np.empty((self.n_points, B), dtype=np.complex128, order="F")
        loss = np.zeros(B, dtype=np.float64)
        _check(self._lib.cui_born_vjp_host(self._plan, g2.ctypes.data, g2.shape[0], u2.ctypes.data, u2.shape[0],
                                           B, grad.ctypes.data, self.n_points,
                                           loss.ctypes.data_as(C.POINTER(C.c_double))))
        return (grad[:, 0], loss[0]) if vec else (grad, loss)

    def lasso_(self, gamma_cols, u_cols, lam, step: float, n_iter: int, loss=None, stream=None):
        """``n_iter`` proximal-gradient LASSO iterations in place (``cui_born_lasso``).

        ``gamma_cols`` (B, n_points) and ``u_cols`` (B, n_observations) are
        contiguous complex64 device tensors (one object per row), ``lam`` a
        float32 device tensor of B thresholds, ``loss`` an optional float32
        device tensor of B values.  Launches only on ``stream`` (default: the
        current torch stream) and allocates nothing, so it may be captured in a
        CUDA graph.
        """
        import torch
        B = gamma_cols.shape[0]
        st = stream if stream is not None else torch.cuda.current_stream(gamma_cols.device).cuda_stream
        _check(self._lib.cui_born_lasso(self._plan, u_cols.data_ptr(), u_cols.shape[1], B, gamma_cols.data_ptr(),
                                        gamma_cols.shape[1], lam.data_ptr(), float(step), int(n_iter),
                                        loss.data_ptr() if loss is not None else None, st))

    def lasso(self, u_meas, lam, step: float, n_iter: int, gamma0=None):
        """Solve ``min 0.5||Phi gamma - u||^2 + lam ||gamma||_1`` per column by ``n_iter``
        proximal-gradient steps from ``gamma0`` (zeros by default); returns ``(gamma, loss)``."""
        import torch
        uc, vec = self._cols(u_meas)
        B = uc.shape[0]
        if gamma0 is None:
            gc = torch.zeros((B, self.n_points), dtype=torch.complex64, device=uc.device)
        else:
            gc, _ = self._cols(gamma0)
            gc = gc.clone()
        lam_t = torch.as_tensor(lam, dtype=torch.float32, device=uc.device).reshape(-1).expand(B).contiguous()
        loss = torch.empty(B, dtype=torch.float32, device=uc.device)
        self.lasso_(gc, uc, lam_t, step, n_iter, loss)
        g = gc.t()
        return (g[:, 0], loss[0]) if vec else (g, loss)

    def energy_rx(self):
        """Received energies ``||Phi e_p||^2`` of every grid point (``cui_born_energy_rx``,
        ``operator_born.m:718-859``): a float32 CUDA tensor of N_points values."""
        import torch
        out = torch.empty(self.n_points, dtype=torch.float32, device="cuda")
        _check(self._lib.cui_born_energy_rx(self._plan, out.data_ptr(), torch.cuda.current_stream().cuda_stream))
        return out

    def omp(self, y, n_atoms_max: int, rel_rmse: float = 0.0):
        """Orthogonal matching pursuit (``cui_born_omp``, ``omp.m:161-200``) on one measured
        column ``y`` (CUDA complex64, N_obs values): returns ``(atoms, coefficients,
        rel_residuals)`` as numpy arrays of the number of atoms taken."""
        import torch
        yc = y.reshape(-1).contiguous()
        atoms = (C.c_int64 * n_atoms_max)()
        coeff = np.zeros(n_atoms_max, dtype=np.complex64)
        res = (C.c_float * n_atoms_max)()
        n = C.c_int32(0)
        _check(self._lib.cui_born_omp(self._plan, yc.data_ptr(), int(n_atoms_max), float(rel_rmse), atoms,
                                      coeff.ctypes.data, res, C.byref(n), torch.cuda.current_stream().cuda_stream))
        k = n.value
        return np.array(atoms[:k], dtype=np.int64), coeff[:k].copy(), np.array(res[:k], dtype=np.float32)

    def cosamp(self, y, sparsity: int, n_iter_max: int, rel_rmse: float = 0.0):
        """Compressive sampling matching pursuit (``cui_born_cosamp``, ``cosamp.m:174-272``) on
        one measured column ``y`` (CUDA complex64, N_obs values): returns ``(atoms,
        coefficients, rel_residuals)``; atoms and coefficients hold the final ``sparsity``
        atoms, largest coefficient first, and ``rel_residuals`` one value per iteration run."""
        import torch
        yc = y.reshape(-1).contiguous()
        atoms = (C.c_int64 * sparsity)()
        coeff = np.zeros(sparsity, dtype=np.complex64)
        res = (C.c_float * max(1, n_iter_max))()
        n = C.c_int32(0)
        _check(self._lib.cui_born_cosamp(self._plan, yc.data_ptr(), int(sparsity), int(n_iter_max), float(rel_rmse),
                                         atoms, coeff.ctypes.data, res, C.byref(n),
                                         torch.cuda.current_stream().cuda_stream))
        return np.array(atoms[:], dtype=np.int64), coeff, np.array(res[:n.value], dtype=np.float32)

    def norm_estimate(self, n_iter: int = 20, seed: int = 0) -> float:
        """||Phi||_2^2 by power iteration on Phi^H Phi (device applies)."""
        import torch
        gen = torch.Generator(device="cuda").manual_seed(seed)
        x = torch.randn((self.n_points, 1), dtype=torch.float32, device="cuda", generator=gen).to(torch.complex64)
        x = x / x.norm()
        lam = 0.0
        for _ in range(n_iter):
            y = self.adjoint(self.forward(x))
            # in FP64: the squares of a small operator's entries (3D setups: |Phi^H Phi x| ~ 1e-25) underflow FP32
            lam = float(torch.linalg.vector_norm(y.to(torch.complex128)))
            x = y / lam
        return lam


def _autograd():
    import torch

    class BornForward(torch.autograd.Function):
        """``u = Phi gamma`` with the hand-written adjoint as its backward.

        For the linear map ``Phi`` PyTorch's complex convention gives the
        input gradient ``Phi^H * grad_u``, which is exactly
        ``cui_born_adjoint``.
        """

        @staticmethod
        def forward(ctx, gamma, op: OperatorBorn):
            ctx.op = op
            return op.forward(gamma)

        @staticmethod
        def backward(ctx, grad_u):
            return ctx.op.adjoint(grad_u.contiguous()), None

    return BornForward


try:  # torch is plumbing for device memory and autograd, not a requirement of the C-ABI
    BornForward = _autograd()
except ImportError:  # pragma: no cover
    BornForward = None


def born_forward(gamma, op: OperatorBorn):
    """Differentiable forward apply (``torch.autograd``)."""
    return BornForward.apply(gamma, op)


def setup_desc(*, n_points_axis: Sequence[int], delta_axis: Sequence[float], z_start: float,
               n_elements_axis: Sequence[int], pitch_axis: Sequence[float], width_axis: Sequence[float],
               n_face_axis: Sequence[int], absorption: dict, f_unique, waves,
               aa_tx_beta: Optional[float] = 0.5, aa_rx_beta: Optional[float] = 0.5, device: int = 0,
               face_apodization=None, lens_focus_axis: Optional[Sequence[float]] = None, lens_c: float = 0.0):
    """``cui_born_setup_desc`` of a discretised setup and the arrays it points into (keep them
    alive while the descriptor is used).

    ``absorption``: ``{"kind": "none"|"time_causal", "c", "constant_db", "slope_db", "exponent",
    "f_ref", "dispersion"}``.  ``waves``: objects or dicts with ``f_idx`` (0-based global
    frequency indices), ``v_d`` ``(F_w, E)`` normal velocities and ``mixes`` (``f_idx``,
    ``active``, ``response`` ``(F_mix, n_active)`` receive responses).  ``aa_*_beta=None``
    switches an anti-aliasing filter off.

    Face weights (``face.m:234-285``): ``face_apodization`` holds the apodization at the
    ``prod(n_face_axis)`` face points, first axis fastest (None: uniform);
    ``lens_focus_axis`` the lens's axial focus per face axis in metres (None, 0 or inf: no
    focusing along that axis); ``lens_c`` the lens's speed of sound (0: 1540 m/s).
    """
    keep = []
    d = SetupDesc()
    nd = len(n_points_axis)
    d.n_dims = nd
    for k in range(nd):
        d.n_points_axis[k] = int(n_points_axis[k])
        d.delta_axis[k] = float(delta_axis[k])
    for k in range(nd - 1):
        d.n_elements_axis[k] = int(n_elements_axis[k])
        d.pitch_axis[k] = float(pitch_axis[k])
        d.width_axis[k] = float(width_axis[k])
        d.n_face_axis[k] = int(n_face_axis[k])
    d.z_start = float(z_start)
    a = AbsorptionDesc()
    a.kind = {"none": 0, "time_causal": 1}[absorption.get("kind", "none")]
    a.c = float(absorption.get("c", 1500.0))
    a.constant_db = float(absorption.get("constant_db", 0.0))
    a.slope_db = float(absorption.get("slope_db", 0.0))
    a.exponent = float(absorption.get("exponent", 1.0))
    a.f_ref = float(absorption.get("f_ref", 4e6))
    a.dispersion = int(bool(absorption.get("dispersion", True)))
    d.absorption = a
    d.aa_tx_beta = -1.0 if aa_tx_beta is None else float(aa_tx_beta)
    d.aa_rx_beta = -1.0 if aa_rx_beta is None else float(aa_rx_beta)
    f = np.ascontiguousarray(np.asarray(f_unique, dtype=np.float64))
    keep.append(f)
    d.n_f_unique = len(f)
    d.f_unique = f.ctypes.data_as(C.POINTER(C.c_double))
    wv = (WaveDesc * len(waves))()
    for w, wave in enumerate(waves):
        f_idx = _i32(np.asarray(_get(wave, "f_idx")) + 1)
        v_d = _c128_f(_get(wave, "v_d"))
        mixes_in = list(_get(wave, "mixes"))
        keep += [f_idx, v_d]
        wv[w].n_f = len(f_idx)
        wv[w].indices_f_to_unique = f_idx.ctypes.data_as(C.POINTER(C.c_int32))
        wv[w].v_d = v_d.ctypes.data
        wv[w].n_mixes = len(mixes_in)
        wv[w].mixes = _mix_array(mixes_in, "response", keep)
    d.n_measurements = len(waves)
    d.waves = wv
    keep.append(wv)
    d.device = int(device)
    if face_apodization is not None:
        fa = np.ascontiguousarray(np.asarray(face_apodization, dtype=np.float64).reshape(-1, order="F"))
        nq = int(np.prod([max(1, int(n_face_axis[k])) for k in range(nd - 1)]))
        if fa.size != nq:
            raise CuiError(1, f"face_apodization has {fa.size} values, the face has {nq} points")
        keep.append(fa)
        d.face_apodization = fa.ctypes.data_as(C.POINTER(C.c_double))
    for k, v in enumerate(lens_focus_axis or ()):
        d.lens_focus_axis[k] = float(v)
    d.lens_c = float(lens_c)
    return d, keep


def setup_hash(**setup) -> str:
    """Hash of the setup fields the device tables depend on (``cui_born_setup_hash``): the
    16-hex-digit name part of the table-cache file.  Needs no GPU."""
    d, keep = setup_desc(**setup)
    out = C.create_string_buffer(17)
    _check(load_library().cui_born_setup_hash(C.byref(d), out))
    return out.value.decode()
