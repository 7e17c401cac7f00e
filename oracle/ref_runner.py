"""MEX gateways run on the host: the reference's ``combined_quick_gpu(operator_born, mode, x)``.

TEST INFRASTRUCTURE ONLY: it pins the oracle (and, through fixtures, the device path) to the
reference's own code.  ``oracle/ref_mex/build.py`` compiles ``+scattering/combined_quick_gpu.cu``
unchanged against host stand-ins of the MEX runtime, the CUDA runtime and cuBLAS
(``oracle/_ref/libref_combined_quick_gpu.so``).  This module builds the ``operator_born`` object
that the gateway reads (``combined_quick_gpu.cu:203-393`` and ``:817-823``) from an
:class:`oracle.born_oracle.OperatorTables` and calls the gateway:

* ``sequence.size``, ``sequence.setup`` (class ``setup_grid_symmetric``, with
  ``indices_grid_FOV_shift`` and ``xdc_array.N_elements``), ``indices_measurement_sel``;
* ``sequence.settings(m).rx(mix).indices_active`` and ``.indices_f_to_unique{mix}``;
* ``sequence.indices_f_to_unique{m}``, ``sequence.prefactors{m}(mix).samples.values``;
* ``options.momentary.gpu`` (class ``gpu_active``, ``index`` 0);
* ``sequence.h_ref.samples.values`` and ``incident_waves(m).p_incident.samples.values``.

All indices are 1-based doubles and all matrices column-major, as MATLAB passes them.
Requires the symmetric representation (``h_ref`` + ``shift``), i.e. a field of view at least as
wide as the array; narrower ones have no valid ``indices_grid_FOV_shift`` in the reference.
The object also carries the grid geometry (``setup.FOV.shape.grid.N_points_axis``,
``setup.xdc_array.N_elements_axis``, ``setup.N_points_per_pitch_axis``) that this library's own
MEX gateways (``comp_ui_toolbox_gb300/mex/``) read; ``ReferenceGateway(path)`` loads any gateway
linked with ``oracle/ref_mex/mex_stub.cpp``.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_ref" / "libref_combined_quick_gpu.so"


class RefMexError(RuntimeError):
    def __init__(self, ident: str, message: str):
        super().__init__(f"{ident}: {message}")
        self.ident = ident
        self.message = message


def available() -> bool:
    return LIB_PATH.exists()


class ReferenceGateway:
    def __init__(self, path: Path = LIB_PATH):
        lib = C.CDLL(str(path))
        vp = C.c_void_p
        lib.ref_new_object.restype = vp
        lib.ref_new_object.argtypes = [C.c_char_p, C.c_size_t]
        lib.ref_new_cell.restype = vp
        lib.ref_new_cell.argtypes = [C.c_size_t]
        lib.ref_new_double.restype = vp
        lib.ref_new_double.argtypes = [C.c_size_t, C.c_size_t, C.c_int, vp]
        lib.ref_set_prop.argtypes = [vp, C.c_size_t, C.c_char_p, vp]
        lib.ref_set_cell.argtypes = [vp, C.c_size_t, vp]
        lib.ref_call.argtypes = [vp, vp, vp, C.c_int, C.POINTER(vp), C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t]
        lib.ref_dims.argtypes = [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_int)]
        lib.ref_read.argtypes = [vp, vp]
        lib.ref_call_args.argtypes = [vp, C.c_int, C.POINTER(vp), C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t]
        if hasattr(lib, "ref_kernel_launches"):
            lib.ref_kernel_launches.restype = C.c_int
        self.lib = lib

    # ---- nodes -------------------------------------------------------------------------
    def obj(self, cls: str, n: int = 1):
        return self.lib.ref_new_object(cls.encode(), n)

    def cell(self, items):
        c = self.lib.ref_new_cell(len(items))
        for i, it in enumerate(items):
            self.lib.ref_set_cell(c, i, it)
        return c

    def dbl(self, a, force_complex: bool = False):
        a = np.asarray(a)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        elif a.ndim == 1:
            a = a.reshape(-1, 1)
        m, n = a.shape
        cplx = force_complex or np.iscomplexobj(a)
        buf = np.asfortranarray(a.astype(np.complex128 if cplx else np.float64))
        flat = buf.reshape(-1, order="F")
        data = np.ascontiguousarray(flat.view(np.float64) if cplx else flat)
        return self.lib.ref_new_double(m, n, int(cplx), data.ctypes.data)

    def set(self, node, name: str, value, index: int = 0):
        if self.lib.ref_set_prop(node, index, name.encode(), value) != 0:
            raise RuntimeError(f"cannot set property {name}")

    def samples(self, values):
        """An object whose ``samples.values`` is the complex matrix ``values``."""
        s = self.obj("processing.signal_matrix")
        self.set(s, "values", self.dbl(values, force_complex=True))
        f = self.obj("processing.field")
        self.set(f, "samples", s)
        return f

    # ---- the operator --------------------------------------------------------------------
    def operator(self, op, gpu_class: str = "scattering.options.gpu_active",
                 setup_class: str = "scattering.sequences.setups.setup_grid_symmetric"):
        if op.h_ref is None or op.shift is None:
            raise ValueError("the reference gateway needs the symmetric representation (h_ref + shift)")
        P = op.setup.n_points
        E = op.setup.n_elements
        W = len(op.measurements)
        ob = self.obj("scattering.operator_born")
        seq = self.obj("scattering.sequences.sequence")
        self.set(ob, "sequence", seq)
        self.set(seq, "size", self.dbl(np.array([[op.n_observations, P]], dtype=float)))
        setup = self.obj(setup_class)
        self.set(setup, "indices_grid_FOV_shift", self.dbl(np.asarray(op.shift, dtype=float)))
        xdc = self.obj("scattering.sequences.setups.transducers.array_planar_regular_orthogonal")
        self.set(xdc, "N_elements", self.dbl(float(E)))
        self.set(xdc, "N_elements_axis", self.dbl(np.asarray(op.setup.n_elements_axis, dtype=float)))
        self.set(setup, "xdc_array", xdc)
        # grid geometry (not read by the reference's gateway; read by this library's gateways)
        self.set(setup, "N_points_per_pitch_axis", self.dbl(np.asarray(op.setup.ppp_axis, dtype=float).reshape(1, -1)))
        grid = self.obj("math.grid_regular_orthogonal")
        self.set(grid, "N_points_axis", self.dbl(np.asarray(op.setup.n_points_axis, dtype=float).reshape(1, -1)))
        shape = self.obj("scattering.sequences.setups.geometry.orthotope")
        self.set(shape, "grid", grid)
        fov = self.obj("scattering.sequences.setups.fields_of_view.field_of_view")
        self.set(fov, "shape", shape)
        self.set(setup, "FOV", fov)
        self.set(seq, "setup", setup)
        self.set(ob, "indices_measurement_sel", self.dbl(np.arange(1, W + 1, dtype=float).reshape(1, -1)))
        settings = self.obj("scattering.sequences.settings.setting", W)
        prefs, f_meas, incident = [], [], self.obj("scattering.sequences.syntheses.incident_wave", W)
        for w, meas in enumerate(op.measurements):
            rx = self.obj("scattering.sequences.settings.controls.rx", len(meas.mixes))
            pm = self.obj("processing.signal_matrix", len(meas.mixes))
            for m, mix in enumerate(meas.mixes):
                self.set(rx, "indices_active", self.dbl(np.asarray(mix.active, dtype=float).reshape(1, -1) + 1),
                         index=m)
                sv = self.obj("physical_values.volt")
                self.set(sv, "values", self.dbl(mix.pref, force_complex=True))
                self.set(pm, "samples", sv, index=m)
            self.set(settings, "rx", rx, index=w)
            self.set(settings, "indices_f_to_unique",
                     self.cell([self.dbl(np.asarray(mix.f_idx, dtype=float) + 1) for mix in meas.mixes]), index=w)
            prefs.append(pm)
            f_meas.append(self.dbl(np.asarray(meas.f_idx, dtype=float) + 1))
            self.set(incident, "p_incident", self.samples(meas.p_incident), index=w)
        self.set(seq, "settings", settings)
        self.set(seq, "indices_f_to_unique", self.cell(f_meas))
        self.set(seq, "prefactors", self.cell(prefs))
        self.set(seq, "h_ref", self.samples(op.h_ref))
        self.set(ob, "incident_waves", incident)
        gpu = self.obj(gpu_class)
        self.set(gpu, "index", self.dbl(0.0))
        mom = self.obj("scattering.options.momentary")
        self.set(mom, "gpu", gpu)
        opts = self.obj("scattering.options")
        self.set(opts, "momentary", mom)
        self.set(ob, "options", opts)
        return ob

    def call(self, op_node, mode, x, nrhs: int = 3) -> np.ndarray:
        """``combined_quick_gpu(op, mode, x)`` with ``mode`` and ``x`` given as values (numbers or
        arrays); raises :class:`RefMexError` with the gateway's error identifier."""
        m = np.asarray(mode)
        return self.call_nodes(op_node, self.dbl(m if np.iscomplexobj(m) else m.astype(float)), self.dbl(np.asarray(x)), nrhs)

    def call_nodes(self, op_node, mode_node, x_node, nrhs: int = 3) -> np.ndarray:
        """The same with every argument given as a node (``obj``, ``cell``, ``dbl``)."""
        return self.call_args([op_node, mode_node, x_node], nrhs)

    def call_args(self, nodes, nrhs: int | None = None) -> np.ndarray:
        """A gateway call with any number of input nodes and one output."""
        arr = (C.c_void_p * max(1, len(nodes)))(*nodes)
        out = C.c_void_p()
        eid, emsg = C.create_string_buffer(256), C.create_string_buffer(512)
        n = len(nodes) if nrhs is None else nrhs
        if self.lib.ref_call_args(arr, n, C.byref(out), eid, 256, emsg, 512) != 0:
            raise RefMexError(eid.value.decode(), emsg.value.decode())
        m, n, c = C.c_size_t(), C.c_size_t(), C.c_int()
        if self.lib.ref_dims(out, C.byref(m), C.byref(n), C.byref(c)) != 0:
            raise RuntimeError("gateway returned no matrix")
        buf = np.empty(m.value * n.value * (2 if c.value else 1), dtype=np.float64)
        self.lib.ref_read(out, buf.ctypes.data)
        vals = buf.view(np.complex128) if c.value else buf
        return vals.reshape((m.value, n.value), order="F")

    def reset(self):
        """Free every node built so far."""
        self.lib.ref_reset()


def forward(op, gamma: np.ndarray, gateway: ReferenceGateway | None = None) -> np.ndarray:
    g = gateway or ReferenceGateway()
    return g.call(g.operator(op), 1, np.asarray(gamma))


def adjoint(op, u: np.ndarray, gateway: ReferenceGateway | None = None) -> np.ndarray:
    g = gateway or ReferenceGateway()
    return g.call(g.operator(op), 2, np.asarray(u))
