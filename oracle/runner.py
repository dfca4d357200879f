"""Python drivers for the oracle libraries — TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional

import numpy as np

from meraxes_gb300.params import GRID_NAMES, MxGlobals, MxGrids, ReionParams

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libmxoracle.so")
# single-precision transforms (the reference's fftwf precision), for CPU timing
TIMING_LIB = os.path.join(ORACLE_DIR, "_build", "libmxoracle_f32.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libmxref.so")
REF_SRC = os.environ.get("MX_REFERENCE_SRC", "/root/reference/src")


def build_oracle(force: bool = False, timing: bool = False) -> str:
    lib, target = (TIMING_LIB, "timing") if timing else (ORACLE_LIB, "oracle")
    if force or not os.path.exists(lib) or _stale(lib, ["mx_oracle.c", "mx_numerics.c", "mx_oracle.h",
                                                        "mx_numerics.h"]):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, target], check=True)
    return lib


def ref_available() -> bool:
    return os.path.isdir(os.path.join(REF_SRC, "core"))


def build_ref(force: bool = False) -> Optional[str]:
    if not ref_available():
        return None
    if force or not os.path.exists(REF_LIB) or _stale(REF_LIB, ["ref_driver.c", "ref_shims.c", "mx_numerics.c"]):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref", f"REF_SRC={REF_SRC}"], check=True)
    return REF_LIB


def _stale(lib: str, srcs) -> bool:
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(os.path.join(ORACLE_DIR, s)) > t for s in srcs)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleBackend:
    """The C restatement, operating in place on a dict of numpy grids."""

    kind = "port"

    def __init__(self, params: ReionParams, redshifts, tables_dir: str, timing: bool = False):
        self.lib = ctypes.CDLL(build_oracle(timing=timing))
        L = self.lib
        L.mxo_create.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
        L.mxo_destroy.argtypes = [ctypes.c_void_p]
        L.mxo_set_redshifts.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.mxo_n_sfr_histories.argtypes = [ctypes.c_void_p]
        for fn in ("mxo_find_HII_bubbles", "mxo_ComputeTs", "mxo_delta_T"):
            getattr(L, fn).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.mxo_last_margin.argtypes = [ctypes.c_void_p]
        L.mxo_last_margin.restype = ctypes.POINTER(ctypes.c_float)
        L.mxo_last_freq_tables.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.mxo_last_freq_tables.restype = ctypes.POINTER(ctypes.c_double)
        L.mxo_recombination_rate_splined.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        L.mxo_recombination_rate_splined.restype = ctypes.c_double
        L.mxo_get_Ts.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
        L.mxo_get_Ts.restype = ctypes.c_double
        L.mxo_construct_baryon_grids.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6 + \
            [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.mxo_calculate_Mvir_crit.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 6 + [ctypes.c_void_p] * 3
        L.mxo_lightcone_init.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.mxo_lightcone_init.restype = ctypes.c_longlong
        L.mxo_construct_lightcone.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 4
        L.mxo_last_velocity_gradient.argtypes = [ctypes.c_void_p]
        L.mxo_last_velocity_gradient.restype = ctypes.POINTER(ctypes.c_float)
        L.mxo_power_spectrum.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.mxo_set_timing_sample.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.mxo_phase_times.argtypes = [ctypes.c_void_p]
        L.mxo_phase_times.restype = ctypes.POINTER(ctypes.c_double)
        self.params = params
        self._pc = params.to_ctypes()
        self.ctx = ctypes.c_void_p()
        rc = L.mxo_create(ctypes.byref(self._pc), tables_dir.encode(), ctypes.byref(self.ctx))
        if rc != 0:
            raise RuntimeError(f"mxo_create failed ({rc})")
        zz = (ctypes.c_double * len(redshifts))(*redshifts)
        L.mxo_set_redshifts(self.ctx, zz, len(redshifts))
        self.n_sfr_histories = L.mxo_n_sfr_histories(self.ctx)

    def close(self):
        if self.ctx:
            self.lib.mxo_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _grids(state: Dict[str, np.ndarray]) -> MxGrids:
        g = MxGrids()
        for n in GRID_NAMES:
            a = state.get(n)
            if a is not None:
                assert a.dtype == np.float32 and a.flags.c_contiguous, n
                setattr(g, n, a.ctypes.data)
        return g

    def _call(self, fn: str, snapshot: int, state) -> Dict[str, float]:
        g = self._grids(state)
        out = MxGlobals()
        rc = getattr(self.lib, fn)(self.ctx, snapshot, ctypes.byref(g), ctypes.byref(out))
        if rc != 0:
            raise RuntimeError(f"{fn} failed ({rc})")
        return out.as_dict()

    def find_HII_bubbles(self, snapshot: int, state) -> Dict[str, float]:
        return self._call("mxo_find_HII_bubbles", snapshot, state)

    def ComputeTs(self, snapshot: int, state) -> Dict[str, float]:
        return self._call("mxo_ComputeTs", snapshot, state)

    def delta_T(self, snapshot: int, state) -> Dict[str, float]:
        return self._call("mxo_delta_T", snapshot, state)

    def construct_baryon_grids(self, snapshot: int, gals: Dict[str, np.ndarray], state, bh=(0, 0.0, 0.0)):
        """construct_baryon_grids on galaxy arrays (pos [n,3] float32, type int32,
        fesc_gsm / gross_sm / bhm / ebhm float64); writes stars, weighted_sfr,
        sfr and sfr_histories of `state` in place."""
        n = len(gals["type"])
        g = self._grids(state)
        rc = self.lib.mxo_construct_baryon_grids(
            self.ctx, snapshot, n, _ptr(gals["pos"]), _ptr(gals["type"]), _ptr(gals["fesc_gsm"]),
            _ptr(gals["gross_sm"]), _ptr(gals.get("bhm")), _ptr(gals.get("ebhm")), bh[0], bh[1], bh[2],
            ctypes.byref(g))
        assert rc == 0, rc

    def calculate_Mvir_crit(self, redshift: float, sm, J_21_at_ion, z_at_ion) -> np.ndarray:
        out = np.zeros_like(J_21_at_ion, dtype=np.float32)
        self.lib.mxo_calculate_Mvir_crit(self.ctx, redshift, *sm, _ptr(J_21_at_ion), _ptr(z_at_ion), _ptr(out))
        return out

    def lightcone_init(self, end_redshift: float, last_output_snap: int):
        """Initialise_ConstructLightcone: (LightconeLength, EndSnapshotLightcone)."""
        e = ctypes.c_int()
        n = self.lib.mxo_lightcone_init(self.ctx, end_redshift, last_output_snap, ctypes.byref(e))
        return int(n), e.value

    def construct_lightcone(self, snapshot: int, delta_T, delta_T_prev, lightcone, lightcone_z):
        """ConstructLightcone, in place on delta_T_prev, lightcone and lightcone_z."""
        rc = self.lib.mxo_construct_lightcone(self.ctx, snapshot, _ptr(delta_T), _ptr(delta_T_prev), _ptr(lightcone),
                                              _ptr(lightcone_z))
        assert rc == 0

    def velocity_gradient(self) -> Optional[np.ndarray]:
        """dv/dx (REAL layout) of the last delta_T with peculiar velocities."""
        ptr = self.lib.mxo_last_velocity_gradient(self.ctx)
        if not ptr:
            return None
        D = self.params.grid_dim
        a = np.ctypeslib.as_array(ptr, shape=(D * D * 2 * (D // 2 + 1),)).reshape(D, D, -1)
        return np.ascontiguousarray(a[:, :, :D])

    def power_spectrum(self, delta_T: np.ndarray):
        """Compute_PS of a REAL delta_T grid: (k, P, error) per k bin."""
        p = self.params
        out = [np.zeros(64, np.float32) for _ in range(3)]
        d = np.ascontiguousarray(delta_T, dtype=np.float32)
        n = self.lib.mxo_power_spectrum(p.grid_dim, p.box_size, p.hubble_h, _ptr(d), *(_ptr(a) for a in out), 64)
        assert n > 0
        return tuple(a[:n].copy() for a in out)

    PHASES = ("forward", "radii", "n_radii", "fhb_post", "shells", "n_shells", "tables", "evolve", "evolve_frac",
              "ts_post", "n_radii_run", "n_shells_run", "shell_copies")

    def set_timing_sample(self, max_radii: int = 0, max_shells: int = 0, cell_div: int = 1):
        """Bounds the work of the next calls for CPU timing (their grids are
        then not the step's results); zeros switch the limits off."""
        self.lib.mxo_set_timing_sample(self.ctx, max_radii, max_shells, cell_div)

    def phase_times(self) -> Dict[str, float]:
        p = self.lib.mxo_phase_times(self.ctx)
        return {n: float(p[i]) for i, n in enumerate(self.PHASES)}

    def margin(self) -> np.ndarray:
        """[2, D, D, D]: first-crossing margin and all-radii margin."""
        D = self.params.grid_dim
        p = self.lib.mxo_last_margin(self.ctx)
        return np.ctypeslib.as_array(p, shape=(2, D, D, D)).copy()

    def freq_tables(self) -> np.ndarray:
        n = ctypes.c_int()
        p = self.lib.mxo_last_freq_tables(self.ctx, ctypes.byref(n))
        return np.ctypeslib.as_array(p, shape=(3, 14, n.value)).copy()

    def step(self, snapshot: int, state) -> Dict[str, float]:
        """ComputeTs -> find_HII_bubbles -> delta_T (dracarys.c:352-390)."""
        out: Dict[str, float] = {}
        if self.params.flag_spin_temp:
            out.update(self.ComputeTs(snapshot, state))
        out.update({k: v for k, v in self.find_HII_bubbles(snapshot, state).items()
                    if k in ("volume_weighted_global_xH", "volume_weighted_global_J_21", "mass_weighted_global_xH",
                             "n_radii")})
        if self.params.flag_21cm:
            out["volume_ave_Tb"] = self.delta_T(snapshot, state)["volume_ave_Tb"]
        return out


class RefBackend:
    """The reference's own sources (compiled with shims); one instance per
    process because the reference keeps its state in globals."""

    kind = "reference"
    _instance = None

    def __init__(self, params: ReionParams, redshifts, tables_dir: str):
        lib = build_ref()
        if lib is None:
            raise RuntimeError("reference tree not available")
        self.lib = ctypes.CDLL(lib, mode=ctypes.RTLD_LOCAL)
        L = self.lib
        L.mxref_init.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_char_p]
        L.mxref_grid.argtypes = [ctypes.c_char_p]
        L.mxref_grid.restype = ctypes.POINTER(ctypes.c_float)
        L.mxref_globals.argtypes = [ctypes.c_void_p]
        L.mxref_stored_fcoll.restype = ctypes.c_double
        L.mxref_splined_recombination_rate.argtypes = [ctypes.c_double, ctypes.c_double]
        L.mxref_splined_recombination_rate.restype = ctypes.c_double
        L.mxref_power_spectrum.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int]
        L.mxref_construct_baryon_grids.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6 + \
            [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.mxref_calculate_Mvir_crit.argtypes = [ctypes.c_double] * 6 + [ctypes.c_void_p] * 3
        L.mxref_lightcone_init.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.mxref_lightcone_init.restype = ctypes.c_longlong
        L.mxref_construct_lightcone.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
        self.params = params
        self._pc = params.to_ctypes()
        zz = (ctypes.c_double * len(redshifts))(*redshifts)
        L.mxref_init(ctypes.byref(self._pc), zz, len(redshifts), tables_dir.encode())
        self.n_sfr_histories = L.mxref_n_sfr_histories()

    def _view(self, name: str, n: int) -> Optional[np.ndarray]:
        p = self.lib.mxref_grid(name.encode())
        if not p:
            return None
        return np.ctypeslib.as_array(p, shape=(n,))

    def _sync_in(self, state):
        for n, a in state.items():
            if n not in GRID_NAMES or a is None:
                continue
            v = self._view(n, a.size)
            if v is not None:
                v[:] = a.ravel()

    def _sync_out(self, state):
        for n, a in state.items():
            if n not in GRID_NAMES or a is None:
                continue
            v = self._view(n, a.size)
            if v is not None:
                a.reshape(-1)[:] = v

    def _run(self, fn, snapshot, state):
        self._sync_in(state)
        getattr(self.lib, fn)(snapshot)
        self._sync_out(state)
        g = MxGlobals()
        self.lib.mxref_globals(ctypes.byref(g))
        d = g.as_dict()
        d["collapse_fraction"] = self.lib.mxref_stored_fcoll(snapshot)
        return d

    def find_HII_bubbles(self, snapshot, state):
        return self._run("mxref_find_HII_bubbles", snapshot, state)

    def construct_baryon_grids(self, snapshot: int, gals, state, bh=(0, 0.0, 0.0)):
        self._sync_in(state)
        self.lib.mxref_construct_baryon_grids(snapshot, len(gals["type"]), _ptr(gals["pos"]), _ptr(gals["type"]),
                                              _ptr(gals["fesc_gsm"]), _ptr(gals["gross_sm"]), _ptr(gals.get("bhm")),
                                              _ptr(gals.get("ebhm")), bh[0], bh[1], bh[2])
        self._sync_out(state)

    def calculate_Mvir_crit(self, redshift: float, sm, J_21_at_ion, z_at_ion) -> np.ndarray:
        out = np.zeros_like(J_21_at_ion, dtype=np.float32)
        self.lib.mxref_calculate_Mvir_crit(redshift, *sm, _ptr(J_21_at_ion), _ptr(z_at_ion), _ptr(out))
        return out

    def lightcone_init(self, end_redshift: float, last_output_snap: int):
        e = ctypes.c_int()
        n = self.lib.mxref_lightcone_init(end_redshift, last_output_snap, ctypes.byref(e))
        return int(n), e.value

    def construct_lightcone(self, snapshot: int, delta_T, delta_T_prev, lightcone, lightcone_z):
        self.lib.mxref_construct_lightcone(snapshot, _ptr(delta_T), _ptr(delta_T_prev), _ptr(lightcone),
                                           _ptr(lightcone_z))

    def power_spectrum(self, delta_T: np.ndarray):
        out = [np.zeros(64, np.float32) for _ in range(3)]
        d = np.ascontiguousarray(delta_T, dtype=np.float32)
        n = self.lib.mxref_power_spectrum(_ptr(d), *(_ptr(a) for a in out), 64)
        assert n > 0, n
        return tuple(a[:n].copy() for a in out)

    def ComputeTs(self, snapshot, state):
        return self._run("mxref_ComputeTs", snapshot, state)

    def delta_T(self, snapshot, state):
        return self._run("mxref_delta_T", snapshot, state)

    def step(self, snapshot, state):
        out = {}
        if self.params.flag_spin_temp:
            out.update(self.ComputeTs(snapshot, state))
        r = self.find_HII_bubbles(snapshot, state)
        for k in ("volume_weighted_global_xH", "volume_weighted_global_J_21", "mass_weighted_global_xH"):
            out[k] = r[k]
        if self.params.flag_21cm:
            out["volume_ave_Tb"] = self.delta_T(snapshot, state)["volume_ave_Tb"]
        return out
