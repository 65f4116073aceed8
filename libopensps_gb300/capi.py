"""ctypes binding of libopensps_gb300.so: the OpenSPS C API entry points of this path.

This is the binding an OpenSPS Python caller would add (the external ``opensps-python`` binds the same symbols
through ctypes/cffi): every function takes and returns what ``include/opensps.h`` declares, and a nonzero status
raises :class:`OpenSPSError` with the library's last-error message.

The library is the product: it must be built (``libopensps_gb300.build.build()``) and there is no fallback; importing
this module without it raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import synthdata

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libopensps_gb300.so"
_lib = None

NBGRAD = 44
DEVICE_PARAMS = ("dust1", "dust2", "dust3", "dust_index", "dust1_index", "frac_nodust", "frac_obrun", "zred",
                 "igm_factor", "sigma_smooth", "dust_tesc", "mwr", "uvb")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# name -> (restype, argtypes): every symbol of include/opensps.h and include/opensps_gb300.h
SIGNATURES = {
    "opensps_clear_error": (None, []),
    "opensps_get_last_error": (None, [_ip, C.c_char_p, C.c_int]),
    "opensps_get_nbgrad": (None, [_ip]),
    "opensps_get_grad_param_name": (None, [C.c_int, C.c_char_p, C.c_int, _ip]),
    "opensps_context_create": (None, [_ip, _ip]),
    "opensps_context_destroy": (None, [C.c_int, _ip]),
    "opensps_context_setup": (None, [C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, _ip]),
    "opensps_context_set_int": (None, [C.c_int, C.c_char_p, C.c_int, _ip]),
    "opensps_context_set_float": (None, [C.c_int, C.c_char_p, C.c_double, _ip]),
    "opensps_context_set_str": (None, [C.c_int, C.c_char_p, C.c_char_p, _ip]),
    "opensps_context_set_fast_mode": (None, [C.c_int, C.c_int, _ip]),
    "opensps_context_get_dims": (None, [C.c_int, _ip, _ip, _ip]),
    "opensps_context_get_nspec": (None, [C.c_int, _ip, _ip]),
    "opensps_context_get_ntfull": (None, [C.c_int, _ip, _ip]),
    "opensps_context_get_nbands": (None, [C.c_int, _ip, _ip]),
    "opensps_context_get_nz": (None, [C.c_int, _ip, _ip]),
    "opensps_context_get_nemline": (None, [C.c_int, _ip, _ip]),
    "opensps_context_get_zsol": (None, [C.c_int, _dp, _ip]),
    "opensps_context_get_lambda": (None, [C.c_int, _dp, _ip]),
    "opensps_context_get_ages": (None, [C.c_int, _dp, _ip]),
    "opensps_context_get_zlegend": (None, [C.c_int, _dp, _ip]),
    "opensps_context_get_emlambda": (None, [C.c_int, _dp, _ip]),
    "opensps_context_set_filters_library": (None, [C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int, _ip]),
    "opensps_context_set_mag_compute": (None, [C.c_int, C.c_int, _ip, _ip]),
    "opensps_context_set_sfh_tab": (None, [C.c_int, C.c_int, _dp, _dp, _dp, _ip]),
    "opensps_context_compute_csp_batch": (None, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, _dp] + [_dp] * 8
                                          + [_ip]),
    "opensps_context_compute_csp_batch_parts": (None, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, _dp]
                                                + [_dp] * 14 + [_ip]),
    "opensps_context_batch_spec_device": (None, [C.c_int, C.POINTER(C.c_void_p), _ip, _ip, _ip, _ip]),
    "opensps_context_batch_spec_host": (None, [C.c_int, C.POINTER(C.c_void_p), _ip, _ip, _ip, _ip]),
    "opensps_context_compute_csp_batch_grad": (None, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, _dp, _dp,
                                                      _dp, _dp, _dp, _dp, _dp] + [_dp] * 8 + [_dp, _dp, _dp, _ip]),
    "opensps_context_compute_csp_batch_grad_rows": (None, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, _dp,
                                                           _dp, _dp, _dp, _dp, _dp, _dp] + [_dp] * 8
                                                    + [_dp, C.c_int, _dp, _dp, _ip]),
    "opensps_context_build_ssp_ops": (None, [C.c_int, C.c_int, _ip]),
    "opensps_context_build_ssp_ops_free_mods": (None, [C.c_int, C.c_int, _ip]),
    "opensps_context_free_ssp_ops": (None, [C.c_int, _ip]),
    "opensps_context_has_ssp_ops": (None, [C.c_int, _ip, _ip]),
    "opensps_context_evaluate_ssp_op": (None, [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _ip]),
    "opensps_gb300_batch_device": (None, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _ip]),
    "opensps_gb300_context_stream": (None, [C.c_int, C.POINTER(C.c_void_p), _ip, _ip]),
    "opensps_gb300_last_launches": (None, [C.c_int, _ip, _ip]),
    "opensps_gb300_ops_last_fold": (None, [C.c_int, _ip, _ip]),
    "opensps_gb300_last_input_in_place": (None, [C.c_int, _ip, _ip]),
    "opensps_gb300_data_table": (None, [C.c_char_p, C.c_char_p, C.c_char_p, _dp, C.c_int, _dp, C.c_longlong,
                                        C.POINTER(C.c_longlong), _ip]),
    "opensps_gb300_spec_mags_noalloc": (None, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _ip]),
    "opensps_gb300_set_profiling": (None, [C.c_int, C.c_int, _ip]),
    "opensps_gb300_kernel_times": (None, [C.c_int, _dp, C.c_int, _ip, _ip]),
    "opensps_gb300_emulator_train": (None, [C.c_int, C.c_char_p, C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_int,
                                            _ip]),
    "opensps_gb300_emulator_load": (None, [C.c_int, C.c_char_p, _ip]),
    "opensps_gb300_emulator_free": (None, [C.c_int, _ip]),
    "opensps_gb300_emulator_info": (None, [C.c_int, _dp, C.c_int, _ip, _ip]),
    "opensps_gb300_emulator_predict": (None, [C.c_int, C.c_int, _dp, C.c_int, _dp, _dp, _dp, _ip, _ip, _ip]),
    "opensps_gb300_emulator_predict_device": (None, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                     C.c_void_p, C.c_void_p, C.c_void_p, _ip, C.c_int, _ip]),
    "opensps_gb300_emulator_set_threshold": (None, [C.c_int, C.c_double, C.c_double, _ip]),
    "opensps_gb300_emulator_init": (None, [C.c_int, C.c_int, _ip]),
    "opensps_gb300_emulator_param_count": (None, [C.POINTER(C.c_longlong)]),
    "opensps_gb300_emulator_params": (None, [C.c_int, C.c_int, C.c_void_p, _ip]),
    "opensps_gb300_emulator_grads": (None, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, _ip]),
}

# the emulator's inputs, in the order of opensps_gb300_emulator_predict
EMU_INPUTS = ("tau", "tage", "logzsol", "dust2", "dust_index", "zred", "sigma_smooth", "imf1", "imf2", "imf3")
EMU_INFO = ("n_train", "n_val", "epochs", "batch", "seed", "t_generate_s", "t_train_s", "val_rms_mag",
            "val_max_mag", "val_p99_mag", "val_flagged_frac", "val_max_unflagged_mag", "pca_explained")


class OpenSPSError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"status {status}: {message}")
        self.status = status
        self.message = message


def library_path() -> Path:
    return _LIB_PATH


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads the C-ABI library (built in-tree); raises if it is missing. No CUDA call is made here."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise OSError(f"{p} is not built: run libopensps_gb300.build.build() (python -c 'import __graft_entry__ as g; "
                      f"g.build()')")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def nbgrad(lib: C.CDLL | None = None) -> int:
    """opensps_get_nbgrad: the rows of params_bar the gradient entry points write."""
    lib = lib or load_library()
    v = C.c_int(0)
    lib.opensps_get_nbgrad(C.byref(v))
    return v.value


def _check(status: C.c_int, lib: C.CDLL):
    if status.value != 0:
        st = C.c_int(0)
        buf = C.create_string_buffer(512)
        lib.opensps_get_last_error(C.byref(st), buf, 512)
        raise OpenSPSError(status.value, buf.value.decode(errors="replace"))


def _names_values(params: dict[str, np.ndarray], n: int):
    names = list(params.keys())
    arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(params[k], dtype=np.float64), (n,))) for k in names]
    c_names = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
    c_vals = (_dp * max(1, len(names)))(*[a.ctypes.data_as(_dp) for a in arrs])
    return len(names), c_names, c_vals, arrs


def data_table(root: str | os.PathLike, kind: str, name: str, lam: np.ndarray | None = None) -> np.ndarray:
    """opensps_gb300_data_table: a standard-format library processed as the context's setup processes it (host only).
    ssp: log L_bol (nz nt,); dust_emission: (2 numin nqpah, nspec) in column order (2 u + c) nqpah + q; agn_torus:
    (9, nspec); filters: (nb, nspec)."""
    lib = load_library()
    g = np.ascontiguousarray(lam if lam is not None else np.zeros(0), dtype=np.float64)
    gp = g.ctypes.data_as(_dp) if g.size else None
    n, st = C.c_longlong(0), C.c_int(0)
    args = (str(root).encode(), kind.encode(), name.encode(), gp, int(g.size))
    lib.opensps_gb300_data_table(*args, None, 0, C.byref(n), C.byref(st))
    _check(st, lib)
    out = np.empty(n.value)
    lib.opensps_gb300_data_table(*args, out.ctypes.data_as(_dp), n.value, C.byref(n), C.byref(st))
    _check(st, lib)
    return out if kind == "ssp" else out.reshape(-1, g.size)


class Context:
    """One OpenSPS context (a handle), set up on the synthetic libraries of the data root."""

    def __init__(self, data_root: str | os.PathLike | None = None, setup: bool = True):
        self.lib = load_library()
        root = Path(data_root) if data_root else synthdata.default_root()
        synthdata.generate(root)
        os.environ["OPENSPS_DATA_HOME"] = str(root)
        h, st = C.c_int(0), C.c_int(0)
        self.lib.opensps_context_create(C.byref(h), C.byref(st))
        _check(st, self.lib)
        self.handle = h.value
        if setup:
            self.setup()

    # -- lifecycle
    def setup(self, isoc: str = "synthetic", spec: str = "synthetic", dust: str = "none"):
        st = C.c_int(0)
        self.lib.opensps_context_setup(-1, isoc.encode(), spec.encode(), dust.encode(), self.handle, C.byref(st))
        _check(st, self.lib)

    def close(self):
        if getattr(self, "handle", 0):
            st = C.c_int(0)
            self.lib.opensps_context_destroy(self.handle, C.byref(st))
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- settings
    def set_int(self, key: str, value: int):
        if key in ("add_dust_emission", "add_agn_dust") and int(value) == 1:
            # the dust emission / AGN torus templates in the data root (written first if missing)
            from . import synth_dust
            gen = synth_dust.generate if key == "add_dust_emission" else synth_dust.generate_agn
            gen(Path(os.environ["OPENSPS_DATA_HOME"]))
        if key == "dust_type" and int(value) in (3, 5):
            # the attenuation libraries in the data root (the synthetic stand-ins written first if missing)
            from . import synth_attenuation
            synth_attenuation.generate(Path(os.environ["OPENSPS_DATA_HOME"]))
        st = C.c_int(0)
        self.lib.opensps_context_set_int(self.handle, key.encode(), int(value), C.byref(st))
        _check(st, self.lib)

    def set_float(self, key: str, value: float):
        st = C.c_int(0)
        self.lib.opensps_context_set_float(self.handle, key.encode(), float(value), C.byref(st))
        _check(st, self.lib)

    def set_str(self, key: str, value: str):
        st = C.c_int(0)
        self.lib.opensps_context_set_str(self.handle, key.encode(), value.encode(), C.byref(st))
        _check(st, self.lib)

    def set_sfh_tab(self, age, sfr, met=None):
        """The tabular SFH of sfh = 3: ages [Gyr] and SFRs [M_sun / yr] (met is not read)."""
        a = np.ascontiguousarray(age, dtype=np.float64)
        s = np.ascontiguousarray(sfr, dtype=np.float64)
        m = None if met is None else np.ascontiguousarray(met, dtype=np.float64)
        st = C.c_int(0)
        self.lib.opensps_context_set_sfh_tab(self.handle, int(a.size), _ptr(a), _ptr(s), _ptr(m), C.byref(st))
        _check(st, self.lib)

    def set_filters_library(self, name: str):
        st = C.c_int(0)
        self.lib.opensps_context_set_filters_library(self.handle, name.encode(), 0, 2, 0, C.byref(st))
        _check(st, self.lib)

    def _get_int(self, fn) -> int:
        v, st = C.c_int(0), C.c_int(0)
        getattr(self.lib, fn)(self.handle, C.byref(v), C.byref(st))
        _check(st, self.lib)
        return v.value

    @property
    def nspec(self) -> int: return self._get_int("opensps_context_get_nspec")
    @property
    def ntfull(self) -> int: return self._get_int("opensps_context_get_ntfull")
    @property
    def nbands(self) -> int: return self._get_int("opensps_context_get_nbands")
    @property
    def nz(self) -> int: return self._get_int("opensps_context_get_nz")
    @property
    def nemline(self) -> int: return self._get_int("opensps_context_get_nemline")

    def _get_arr(self, fn, n) -> np.ndarray:
        out, st = np.empty(n), C.c_int(0)
        getattr(self.lib, fn)(self.handle, _ptr(out), C.byref(st))
        _check(st, self.lib)
        return out

    def wavelengths(self) -> np.ndarray: return self._get_arr("opensps_context_get_lambda", self.nspec)
    def ages(self) -> np.ndarray: return self._get_arr("opensps_context_get_ages", self.ntfull)
    def zlegend(self) -> np.ndarray: return self._get_arr("opensps_context_get_zlegend", self.nz)

    # -- batches
    def csp_batch(self, params: dict, ssp_weights_z: np.ndarray | None = None, ssp_weights: np.ndarray | None = None,
                  spec: bool = True, mass: bool = True, lbol: bool = True) -> dict:
        """compute_csp_batch_grad with no cotangents (the forward batch): weights (n, nz, nt) or (n, nt), or none
        (the context's SFH from the parameters tage, tau, ...; n from the parameter arrays)."""
        if ssp_weights_z is not None:
            w = np.ascontiguousarray(ssp_weights_z, dtype=np.float64)
            n = w.shape[0]
        elif ssp_weights is not None:
            w = np.ascontiguousarray(ssp_weights, dtype=np.float64)
            n = w.shape[0]
        else:
            w = None
            n = max(np.size(v) for v in params.values())
        ns, nb = self.nspec, self.nbands
        k, c_names, c_vals, keep = _names_values(params, n)
        out = {"mags": np.empty((n, nb))}
        if spec: out["spec"] = np.empty((n, ns))
        if mass: out["mass"] = np.empty(n)
        if lbol: out["lbol"] = np.empty(n)
        st = C.c_int(0)
        if ssp_weights_z is not None:
            self.lib.opensps_context_compute_csp_batch_grad(
                self.handle, n, k, c_names, c_vals, None, _ptr(w), None, None, None, None, None,
                _ptr(out["mags"]), _ptr(out.get("spec")), _ptr(out.get("mass")), _ptr(out.get("lbol")), None, None,
                None, None, None, None, None, C.byref(st))
        else:
            self.lib.opensps_context_compute_csp_batch(
                self.handle, n, k, c_names, c_vals, _ptr(w), _ptr(out["mags"]), _ptr(out.get("spec")),
                _ptr(out.get("mass")), _ptr(out.get("lbol")), None, None, None, None, C.byref(st))
        _check(st, self.lib)
        del keep
        return out

    def csp_batch_grad(self, params: dict, ssp_weights_z: np.ndarray | None = None, mags_bar: np.ndarray | None = None,
                       spec_bar: np.ndarray | None = None, mass_bar: np.ndarray | None = None,
                       lbol_bar: np.ndarray | None = None, params_bar_rows: int | None = None,
                       weights_z_bar: bool = True, spec: bool = True, out: dict | None = None,
                       ssp_weights: np.ndarray | None = None, n: int | None = None) -> dict:
        """compute_csp_batch_grad_rows: the forward batch and the reverse pass for the given cotangents (arrays
        (n, nbands), (n, nspec), (n,), (n,)). Weights: ssp_weights_z (n, nz, nt), or ssp_weights (n, nt) blended at
        logzsol, or neither (the context's SFH from the per-model SFH parameters; give n). Returns the forward
        outputs (mags, mass, lbol, and spec unless spec=False), params_bar (n, rows) and weights_z_bar (n, nz, nt)
        with ssp_weights_z, weights_bar (n, nt) otherwise. ``out`` may hold preallocated C-contiguous float64 arrays
        for any of these (e.g. page-locked ones)."""
        w = None if ssp_weights_z is None else np.ascontiguousarray(ssp_weights_z, dtype=np.float64)
        wa = None if ssp_weights is None else np.ascontiguousarray(ssp_weights, dtype=np.float64)
        if w is not None:
            n = w.shape[0]
        elif wa is not None:
            n = wa.shape[0]
        elif n is None:
            raise ValueError("give n with SFH parameters (no weights)")
        ns, nb, nt, nz = self.nspec, self.nbands, self.ntfull, self.nz
        rows = params_bar_rows if params_bar_rows is not None else nbgrad(self.lib)
        k, c_names, c_vals, keep = _names_values(params, n)
        cot = {}
        for name, arr in (("mags_bar", mags_bar), ("spec_bar", spec_bar), ("mass_bar", mass_bar),
                          ("lbol_bar", lbol_bar)):
            cot[name] = None if arr is None else np.ascontiguousarray(arr, dtype=np.float64)
        shapes = {"mags": (n, nb), "mass": (n,), "lbol": (n,), "params_bar": (n, rows)}
        if spec:
            shapes["spec"] = (n, ns)
        if weights_z_bar and w is not None:
            shapes["weights_z_bar"] = (n, nz, nt)
        if weights_z_bar and w is None:
            shapes["weights_bar"] = (n, nt)
        given = out or {}
        res = {}
        for name, shp in shapes.items():
            a = given.get(name)
            if a is None:
                a = np.empty(shp)
            elif a.shape != shp or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"out[{name!r}] must be a C-contiguous float64 array of shape {shp}")
            res[name] = a
        st = C.c_int(0)
        self.lib.opensps_context_compute_csp_batch_grad_rows(
            self.handle, n, k, c_names, c_vals, _ptr(wa), _ptr(w), None, _ptr(cot["mags_bar"]), _ptr(cot["spec_bar"]),
            _ptr(cot["mass_bar"]), _ptr(cot["lbol_bar"]), _ptr(res["mags"]), _ptr(res.get("spec")),
            _ptr(res["mass"]), _ptr(res["lbol"]), None, None, None, None, _ptr(res["params_bar"]), rows,
            _ptr(res.get("weights_bar")), _ptr(res.get("weights_z_bar")), C.byref(st))
        _check(st, self.lib)
        del keep
        return res

    def csp_batch_parts(self, params: dict, ssp_weights: np.ndarray, emlines: bool = True) -> dict:
        """compute_csp_batch_parts: the batch with the intrinsic young and old age sums (weights (n, nt))."""
        w = np.ascontiguousarray(ssp_weights, dtype=np.float64)
        n = w.shape[0]
        ns, nb, nl = self.nspec, self.nbands, self.nemline
        k, c_names, c_vals, keep = _names_values(params, n)
        out = {"mags": np.empty((n, nb)), "spec": np.empty((n, ns)), "mass": np.empty(n), "lbol": np.empty(n),
               "young": np.empty((n, ns)), "old": np.empty((n, ns)), "mass_young": np.empty(n),
               "mass_old": np.empty(n), "lbol_young": np.empty(n), "lbol_old": np.empty(n)}
        if emlines:
            out["emlines"] = np.empty((n, nl))
        st = C.c_int(0)
        self.lib.opensps_context_compute_csp_batch_parts(
            self.handle, n, k, c_names, c_vals, _ptr(w), _ptr(out["mags"]), _ptr(out["spec"]), _ptr(out["mass"]),
            _ptr(out["lbol"]), None, None, _ptr(out.get("emlines")), None, _ptr(out["young"]), _ptr(out["old"]),
            _ptr(out["mass_young"]), _ptr(out["mass_old"]), _ptr(out["lbol_young"]), _ptr(out["lbol_old"]),
            C.byref(st))
        _check(st, self.lib)
        del keep
        return out

    def batch_device(self, n: int, d_params: int, d_wz: int, d_mags: int | None, sync: bool = True):
        """opensps_gb300_batch_device with device pointers (integers, e.g. torch.Tensor.data_ptr())."""
        st = C.c_int(0)
        self.lib.opensps_gb300_batch_device(self.handle, n, C.c_void_p(d_params), C.c_void_p(d_wz),
                                            C.c_void_p(d_mags) if d_mags else None, 1 if sync else 0, C.byref(st))
        _check(st, self.lib)

    def spec_device(self):
        p, ns, n, b, st = C.c_void_p(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.lib.opensps_context_batch_spec_device(self.handle, C.byref(p), C.byref(ns), C.byref(n), C.byref(b),
                                                   C.byref(st))
        _check(st, self.lib)
        return p.value, ns.value, n.value, b.value

    # -- SSP operators (the IMF per model)
    def build_ssp_ops(self, all_metallicities: bool = True):
        """opensps_context_build_ssp_ops over the data root's operator dataset (written first if missing)."""
        from . import synth_ops
        synth_ops.generate(Path(os.environ["OPENSPS_DATA_HOME"]))
        st = C.c_int(0)
        self.lib.opensps_context_build_ssp_ops(self.handle, 1 if all_metallicities else 0, C.byref(st))
        _check(st, self.lib)

    def free_ssp_ops(self):
        st = C.c_int(0)
        self.lib.opensps_context_free_ssp_ops(self.handle, C.byref(st))
        _check(st, self.lib)

    @property
    def has_ssp_ops(self) -> bool:
        h, st = C.c_int(0), C.c_int(0)
        self.lib.opensps_context_has_ssp_ops(self.handle, C.byref(h), C.byref(st))
        _check(st, self.lib)
        return bool(h.value)

    def evaluate_ssp_op(self, imf_params=None, imf_type: int = 2) -> dict:
        """opensps_context_evaluate_ssp_op: one IMF's SSP grid at the context's zmet: mass, lbol (ntfull,) and spec
        (ntfull, nspec)."""
        nt, ns = self.ntfull, self.nspec
        out = {"mass": np.empty(nt), "lbol": np.empty(nt), "spec": np.empty((nt, ns))}
        p = None if imf_params is None else np.ascontiguousarray(imf_params, dtype=np.float64)
        st = C.c_int(0)
        self.lib.opensps_context_evaluate_ssp_op(self.handle, imf_type, _ptr(p), _ptr(out["mass"]), _ptr(out["lbol"]),
                                                 _ptr(out["spec"]), C.byref(st))
        _check(st, self.lib)
        return out

    def spec_mags_noalloc(self, n: int, d_spec: int, d_zred: int, d_mags: int, sync: bool = True):
        """opensps_gb300_spec_mags_noalloc: magnitudes of device spectra (nspec x n floats) at device redshifts (n
        doubles) into d_mags (nbands x n doubles), with no allocation (device pointers as integers)."""
        st = C.c_int(0)
        self.lib.opensps_gb300_spec_mags_noalloc(self.handle, n, C.c_void_p(d_spec), C.c_void_p(d_zred),
                                                 C.c_void_p(d_mags), 1 if sync else 0, C.byref(st))
        _check(st, self.lib)

    def stream(self) -> int:
        s, d, st = C.c_void_p(), C.c_int(), C.c_int()
        self.lib.opensps_gb300_context_stream(self.handle, C.byref(s), C.byref(d), C.byref(st))
        _check(st, self.lib)
        return s.value or 0

    def last_launches(self) -> int:
        return self._get_int("opensps_gb300_last_launches")

    def last_input_in_place(self) -> bool:
        """Whether the last batch read the caller's pageable weights in place (else they were copied)."""
        return bool(self._get_int("opensps_gb300_last_input_in_place"))

    def ops_last_interpolated(self) -> bool:
        """Whether the last batch through the SSP operator took the interpolated fold (else the exact one)."""
        return bool(self._get_int("opensps_gb300_ops_last_fold"))

    def set_profiling(self, on: bool):
        st = C.c_int(0)
        self.lib.opensps_gb300_set_profiling(self.handle, 1 if on else 0, C.byref(st))
        _check(st, self.lib)

    def kernel_times(self) -> list[float]:
        """Mean device ms of the profiled batches' stages: model parameters, weight operand, contraction, bands, FP64 sums
        (and after gradient calls: output and cotangent copies, adjoint, weights GEMMs, weights cotangent)."""
        buf, n, st = np.zeros(10), C.c_int(0), C.c_int(0)
        self.lib.opensps_gb300_kernel_times(self.handle, _ptr(buf), 10, C.byref(n), C.byref(st))
        _check(st, self.lib)
        return buf[:n.value].tolist()

    # -- the learned emulator (include/opensps_gb300.h)
    def emulator_train(self, path: str | os.PathLike | None, n_train: int = 4194304, n_val: int = 32768,
                       epochs: int = 60, batch: int = 8192, seed: int = 1):
        """opensps_gb300_emulator_train on this context's CSP: builds the SSP operators and sets sfh = 4 first."""
        if not self.has_ssp_ops:
            self.build_ssp_ops()
        self.set_int("sfh", 4)
        st = C.c_int(0)
        self.lib.opensps_gb300_emulator_train(self.handle, str(path).encode() if path else None, n_train, n_val,
                                              epochs, batch, seed, C.byref(st))
        _check(st, self.lib)

    def emulator_load(self, path: str | os.PathLike):
        st = C.c_int(0)
        self.lib.opensps_gb300_emulator_load(self.handle, str(path).encode(), C.byref(st))
        _check(st, self.lib)

    def emulator_free(self):
        st = C.c_int(0)
        self.lib.opensps_gb300_emulator_free(self.handle, C.byref(st))
        _check(st, self.lib)

    def emulator_info(self) -> dict:
        buf, n, st = np.zeros(32), C.c_int(0), C.c_int(0)
        self.lib.opensps_gb300_emulator_info(self.handle, _ptr(buf), 32, C.byref(n), C.byref(st))
        _check(st, self.lib)
        return dict(zip(EMU_INFO, buf[:n.value].tolist()))

    def emulator_set_threshold(self, spread_max: float = 0.01, faint: float = 15.0):
        st = C.c_int(0)
        self.lib.opensps_gb300_emulator_set_threshold(self.handle, spread_max, faint, C.byref(st))
        _check(st, self.lib)

    def emulator_predict(self, inputs: dict | np.ndarray, fallback: bool = True, pca: bool = False) -> dict:
        """opensps_gb300_emulator_predict. inputs: a dict of the EMU_INPUTS arrays or an (n, 10) array. Returns mags
        (n, nbands), spread (n,), source (n,) and n_fallback (and pca (n, 64))."""
        if isinstance(inputs, dict):
            x = np.stack([np.asarray(inputs[k], dtype=np.float64) for k in EMU_INPUTS], axis=1)
        else:
            x = np.asarray(inputs, dtype=np.float64)
        x = np.ascontiguousarray(x)
        n, nb = x.shape[0], self.nbands
        out = {"mags": np.empty((n, nb)), "spread": np.empty(n), "source": np.empty(n, dtype=np.int32)}
        if pca:
            out["pca"] = np.empty((n, 64))
        nf, st = C.c_int(0), C.c_int(0)
        self.lib.opensps_gb300_emulator_predict(self.handle, n, _ptr(x), 1 if fallback else 0, _ptr(out["mags"]),
                                                _ptr(out.get("pca")), _ptr(out["spread"]),
                                                out["source"].ctypes.data_as(_ip), C.byref(nf), C.byref(st))
        _check(st, self.lib)
        out["n_fallback"] = nf.value
        return out

    def emulator_predict_device(self, n: int, d_inputs: int, d_mags: int, d_flag: int, d_flagged: int,
                                d_pca: int = 0, d_spread: int = 0, count: bool = True, sync: bool = True) -> int:
        """opensps_gb300_emulator_predict_device on device pointers (integers); returns the flagged count (or -1)."""
        nf, st = C.c_int(0), C.c_int(0)
        self.lib.opensps_gb300_emulator_predict_device(self.handle, n, C.c_void_p(d_inputs), C.c_void_p(d_mags),
                                                       C.c_void_p(d_pca or None), C.c_void_p(d_spread or None),
                                                       C.c_void_p(d_flag), C.c_void_p(d_flagged),
                                                       C.byref(nf) if count else None, 1 if sync else 0, C.byref(st))
        _check(st, self.lib)
        return nf.value if count else -1

    def emulator_init(self, seed: int = 0):
        st = C.c_int(0)
        self.lib.opensps_gb300_emulator_init(self.handle, seed, C.byref(st))
        _check(st, self.lib)

    def emulator_param_count(self) -> int:
        v = C.c_longlong(0)
        self.lib.opensps_gb300_emulator_param_count(C.byref(v))
        return v.value

    def emulator_params(self, values: np.ndarray | None = None) -> np.ndarray:
        """Gets (values None) or sets the FP32 parameters [w0 | wh | w4 | bias]."""
        st = C.c_int(0)
        if values is None:
            buf = np.empty(self.emulator_param_count(), dtype=np.float32)
            self.lib.opensps_gb300_emulator_params(self.handle, 0, C.c_void_p(buf.ctypes.data), C.byref(st))
            _check(st, self.lib)
            return buf
        buf = np.ascontiguousarray(values, dtype=np.float32)
        self.lib.opensps_gb300_emulator_params(self.handle, 1, C.c_void_p(buf.ctypes.data), C.byref(st))
        _check(st, self.lib)
        return buf

    def emulator_grads(self, x_std: np.ndarray, y_std: np.ndarray, loss_weights: np.ndarray):
        """opensps_gb300_emulator_grads: (loss (5,), grads (param_count,)) of the training kernels on one minibatch."""
        x = np.ascontiguousarray(x_std, dtype=np.float32)
        y = np.ascontiguousarray(y_std, dtype=np.float32)
        w = np.ascontiguousarray(loss_weights, dtype=np.float32)
        loss = np.zeros(5, dtype=np.float32)
        g = np.zeros(self.emulator_param_count(), dtype=np.float32)
        st = C.c_int(0)
        self.lib.opensps_gb300_emulator_grads(self.handle, x.shape[0], C.c_void_p(x.ctypes.data),
                                              C.c_void_p(y.ctypes.data), C.c_void_p(w.ctypes.data),
                                              C.c_void_p(loss.ctypes.data), C.c_void_p(g.ctypes.data), C.byref(st))
        _check(st, self.lib)
        return loss, g
