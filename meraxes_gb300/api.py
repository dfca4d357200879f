"""High-level interface of the reionization grid step.

`ReionGridStep` mirrors the reference's entry points (src/core/find_HII_bubbles.c
find_HII_bubbles, src/core/ComputeTs.c ComputeTs,
src/core/BrightnessTemperature.c ComputeBrightnessTemperatureBox): one object
per run holds the parameters, the snapshot redshift list and the device
context; each call takes the grids of one snapshot.

Grids are passed as a dict name -> array in the reference layouts (PADDED for
deltax, stars, weighted_sfr, sfr, N_rec, x_e_box, x_e_box_prev, vel; REAL for
the rest; sfr_histories as [n_slices, padded]).  numpy arrays select the
host-pointer entry points (host<->device copies inside the call); CUDA torch
tensors select the device entry points on torch's current stream.
"""
from __future__ import annotations

import contextlib
import ctypes
from typing import Dict, Optional, Sequence

import numpy as np

from . import _lib
from .params import GRID_NAMES, MxGalaxies, MxGlobals, MxGrids, ReionParams
from .synthetic import TABLES_DIR


def _is_torch_cuda(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


class ReionGridStep:
    def __init__(self, params: ReionParams, redshifts: Sequence[float], tables_dir: str = TABLES_DIR,
                 max_work_bytes: int = 0):
        """max_work_bytes caps the transform work buffer (mx_create_limited);
        0 lets it take up to 45% of the free device memory."""
        self.lib = _lib.load()
        self.params = params
        self._pc = params.to_ctypes()
        self.ctx = ctypes.c_void_p()
        if max_work_bytes:
            rc = self.lib.mx_create_limited(ctypes.byref(self._pc), tables_dir.encode(), int(max_work_bytes),
                                            ctypes.byref(self.ctx))
        else:
            rc = self.lib.mx_create(ctypes.byref(self._pc), tables_dir.encode(), ctypes.byref(self.ctx))
        if rc != 0:
            raise _lib.MxError(rc, self.lib.mx_last_error(None).decode())
        zz = (ctypes.c_double * len(redshifts))(*[float(z) for z in redshifts])
        self._check(self.lib.mx_set_redshifts(self.ctx, zz, len(redshifts)))
        self.redshifts = list(redshifts)
        self.n_sfr_histories = int(self.lib.mx_n_sfr_histories(self.ctx))
        self.last_launches = 0

    # ------------------------------------------------------------------ utils
    @contextlib.contextmanager
    def _stream(self):
        """The CUDA stream of a device call: torch's current stream; or, when
        that is the default stream (handle 0, which the library reads as its
        own non-blocking context stream), a side stream that starts after the
        caller's pending default-stream work and that the default stream then
        waits for."""
        import torch

        cur = torch.cuda.current_stream()
        if cur.cuda_stream != 0:
            yield cur.cuda_stream
            return
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream()
        self._side.wait_stream(cur)
        try:
            yield self._side.cuda_stream
        finally:
            cur.wait_stream(self._side)

    def _check(self, rc: int):
        if rc != 0:
            raise _lib.MxError(rc, self.lib.mx_last_error(self.ctx).decode())

    def close(self):
        if self.ctx:
            self.lib.mx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def filter_radii(self):
        buf = (ctypes.c_double * 1024)()
        n = self.lib.mx_filter_radii(self.ctx, buf, 1024)
        return list(buf[:n])

    def zpass_blocks(self) -> int:
        """Resident blocks per SM the threshold z-pass was tuned for (0: not run)."""
        return int(self.lib.mx_zpass_blocks_per_sm(self.ctx))

    def set_graph(self, on: bool = True):
        """Device steps (step() on CUDA tensors) captured and launched as one
        CUDA graph each (mx_set_step_graph)."""
        self._check(self.lib.mx_set_step_graph(self.ctx, 1 if on else 0))

    def fft_block_sizes(self):
        """Threads per block of the fused x- and y-pass chosen at creation."""
        x, y = ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.mx_fft_block_sizes(self.ctx, ctypes.byref(x), ctypes.byref(y)))
        return x.value, y.value

    def _grids(self, grids: Dict[str, object]):
        g = MxGrids()
        device = None
        for name in GRID_NAMES:
            a = grids.get(name)
            if a is None:
                continue
            if _is_torch_cuda(a):
                if device is False:
                    raise ValueError("mixing host and device grids")
                device = True
                import torch

                if a.dtype != torch.float32 or not a.is_contiguous():
                    raise ValueError(f"{name}: need contiguous float32")
                setattr(g, name, a.data_ptr())
            else:
                if device is True:
                    raise ValueError("mixing host and device grids")
                device = False
                if not isinstance(a, np.ndarray) or a.dtype != np.float32 or not a.flags.c_contiguous:
                    raise ValueError(f"{name}: need C-contiguous float32 numpy array")
                setattr(g, name, a.ctypes.data)
        return g, bool(device)

    def _call(self, name: str, snapshot: int, grids) -> Dict[str, float]:
        g, device = self._grids(grids)
        out = MxGlobals()
        if device:
            import torch

            with self._stream() as stream:
                rc = getattr(self.lib, name + "_device")(self.ctx, snapshot, ctypes.byref(g), ctypes.byref(out),
                                                        ctypes.c_void_p(stream))
        else:
            rc = getattr(self.lib, name)(self.ctx, snapshot, ctypes.byref(g), ctypes.byref(out))
        self._check(rc)
        self.last_launches = out.gpu_launches
        return out.as_dict()

    def profile(self, on: bool = True):
        """Start (clear) or stop per-kernel CUDA-event timing."""
        self._check(self.lib.mx_profile_enable(self.ctx, 1 if on else 0))

    def profile_read(self):
        """{kernel name: (launches, total ms, algorithmic bytes)}."""
        buf = (_lib.MxKernelStat * 64)()
        n = self.lib.mx_profile_read(self.ctx, buf, 64)
        if n < 0:
            self._check(n)
        return {buf[i].name.decode(): (buf[i].launches, buf[i].ms, buf[i].bytes) for i in range(min(n, 64))}

    # --------------------------------------------------------- entry points
    def find_HII_bubbles(self, snapshot: int, grids) -> Dict[str, float]:
        return self._call("mx_find_HII_bubbles", snapshot, grids)

    def ComputeTs(self, snapshot: int, grids) -> Dict[str, float]:
        return self._call("mx_ComputeTs", snapshot, grids)

    def ComputeBrightnessTemperatureBox(self, snapshot: int, grids) -> Dict[str, float]:
        return self._call("mx_ComputeBrightnessTemperatureBox", snapshot, grids)

    def step(self, snapshot: int, grids) -> Dict[str, float]:
        """ComputeTs -> find_HII_bubbles -> brightness temperature."""
        return self._call("mx_step", snapshot, grids)

    def Compute_PS(self, delta_T):
        """21 cm power spectrum of a REAL delta_T grid (numpy array, or a CUDA
        tensor on the current stream): (k [1/Mpc], P [mK^2], error) per bin."""
        n = self.lib.mx_ps_length(self.ctx)
        if n < 0:
            self._check(n)
        out = [np.zeros(n, np.float32) for _ in range(3)]
        ptrs = [o.ctypes.data for o in out]
        if _is_torch_cuda(delta_T):
            import torch

            if delta_T.dtype != torch.float32 or not delta_T.is_contiguous():
                raise ValueError("delta_T: need contiguous float32")
            with self._stream() as stream:
                rc = self.lib.mx_Compute_PS_device(self.ctx, delta_T.data_ptr(), *ptrs, n, ctypes.c_void_p(stream))
        else:
            d = np.ascontiguousarray(delta_T, dtype=np.float32)
            rc = self.lib.mx_Compute_PS(self.ctx, d.ctypes.data, *ptrs, n)
        if rc < 0:
            self._check(rc)
        return tuple(out)

    def lightcone_init(self, end_redshift: float, last_output_snap: int):
        """Initialise_ConstructLightcone: (LightconeLength, EndSnapshotLightcone)."""
        end = ctypes.c_int32()
        n = self.lib.mx_lightcone_init(self.ctx, end_redshift, last_output_snap, ctypes.byref(end))
        if n < 0:
            self._check(int(n))
        return int(n), end.value

    def ConstructLightcone(self, snapshot: int, delta_T, delta_T_prev, lightcone, lightcone_redshifts):
        """Fills this snapshot's slices of `lightcone` ([D][D][length]) and
        `lightcone_redshifts` (numpy, host) and copies delta_T into
        delta_T_prev.  Grids and light cone are numpy arrays or CUDA tensors
        (device family, current stream)."""
        z = lightcone_redshifts
        if not (isinstance(z, np.ndarray) and z.dtype == np.float32 and z.flags.c_contiguous):
            raise ValueError("lightcone_redshifts: need a C-contiguous float32 numpy array")
        if _is_torch_cuda(delta_T):
            import torch

            with self._stream() as stream:
                rc = self.lib.mx_ConstructLightcone_device(self.ctx, snapshot, delta_T.data_ptr(), delta_T_prev.data_ptr(),
                                                           lightcone.data_ptr(), z.ctypes.data, ctypes.c_void_p(stream))
        else:
            for a in (delta_T, delta_T_prev, lightcone):
                if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                    raise ValueError("need C-contiguous float32 numpy arrays")
            rc = self.lib.mx_ConstructLightcone(self.ctx, snapshot, delta_T.ctypes.data, delta_T_prev.ctypes.data,
                                                lightcone.ctypes.data, z.ctypes.data)
        self._check(rc)

    _GALAXY_DTYPES = {"pos": "float32", "type": "int32", "fesc_weighted_gsm": "float64",
                      "gross_stellar_mass": "float64", "black_hole_mass": "float64", "effective_bhm": "float64"}

    def _galaxies(self, galaxies, device: bool):
        g = MxGalaxies()
        n = None
        for name, dt in self._GALAXY_DTYPES.items():
            a = galaxies.get(name)
            if a is None:
                continue
            if device:
                import torch

                if not _is_torch_cuda(a) or a.dtype != getattr(torch, dt) or not a.is_contiguous():
                    raise ValueError(f"{name}: need a contiguous {dt} CUDA tensor")
                ptr = a.data_ptr()
            else:
                if not isinstance(a, np.ndarray) or a.dtype != np.dtype(dt) or not a.flags.c_contiguous:
                    raise ValueError(f"{name}: need a C-contiguous {dt} numpy array")
                ptr = a.ctypes.data
            rows = a.shape[0] if len(a.shape) else 0
            if name == "pos" and tuple(a.shape[1:]) != (3,):
                raise ValueError("pos: need shape [n, 3]")
            if n is not None and rows != n:
                raise ValueError(f"{name}: {rows} galaxies, expected {n}")
            n = rows
            setattr(g, name, ptr)
        g.n = n or 0
        return g

    def construct_baryon_grids(self, snapshot: int, galaxies, grids, flag_bh_feedback: int = 0,
                               bh_limit: float = 0.0, alpha_uv_bh: float = 0.0):
        """construct_baryon_grids: deposits the galaxies (dict of arrays named
        like `mx_galaxies`: pos [n, 3] float32, type int32, the masses float64)
        into grids["stars"], ["weighted_sfr"] and, with the spin temperature,
        ["sfr"] and ["sfr_histories"].  numpy arrays select the host entry
        point; CUDA tensors the device one on torch's current stream."""
        g, device = self._grids(grids)
        gal = self._galaxies(galaxies, device)
        if device:
            import torch

            with self._stream() as stream:
                rc = self.lib.mx_construct_baryon_grids_device(self.ctx, snapshot, ctypes.byref(gal), flag_bh_feedback,
                                                              bh_limit, alpha_uv_bh, ctypes.byref(g),
                                                              ctypes.c_void_p(stream))
        else:
            rc = self.lib.mx_construct_baryon_grids(self.ctx, snapshot, ctypes.byref(gal), flag_bh_feedback, bh_limit,
                                                   alpha_uv_bh, ctypes.byref(g))
        self._check(rc)

    def calculate_Mvir_crit(self, redshift: float, sm_params, J_21_at_ionization, z_at_ionization, Mvir_crit):
        """calculate_Mvir_crit: writes Mvir_crit (REAL) from the ionisation
        history; sm_params = (ReionSMParam_m0, _a, _b, _c, _d)."""
        sm = (ctypes.c_double * 5)(*[float(v) for v in sm_params])
        arrays = (J_21_at_ionization, z_at_ionization, Mvir_crit)
        if _is_torch_cuda(Mvir_crit):
            import torch

            for a in arrays:
                if not _is_torch_cuda(a) or a.dtype != torch.float32 or not a.is_contiguous():
                    raise ValueError("need contiguous float32 CUDA tensors")
            with self._stream() as stream:
                rc = self.lib.mx_calculate_Mvir_crit_device(self.ctx, redshift, sm, *[a.data_ptr() for a in arrays],
                                                            ctypes.c_void_p(stream))
        else:
            for a in arrays:
                if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                    raise ValueError("need C-contiguous float32 numpy arrays")
            rc = self.lib.mx_calculate_Mvir_crit(self.ctx, redshift, sm, *[a.ctypes.data for a in arrays])
        self._check(rc)

    # ------------------------------------------------------- differentiation
    def set_xray(self, lx_gal: float, nu_xray_gal_threshold: float):
        """LXrayGal and NuXrayGalThreshold (E0, eV) for the following calls."""
        self._check(self.lib.mx_set_xray_params(self.ctx, float(lx_gal), float(nu_xray_gal_threshold)))
        self.params.lx_gal = float(lx_gal)
        self.params.nu_xray_gal_threshold = float(nu_xray_gal_threshold)

    def ps_loss(self, delta_T, edges, target, grad: bool = True):
        """Binned power-spectrum loss of a REAL delta_T CUDA tensor (see
        mx_ps_loss_device): (loss, P per bin, dL/d(delta_T) or None)."""
        import torch

        nb = len(target)
        e = (ctypes.c_float * (nb + 1))(*[float(v) for v in edges])
        t = (ctypes.c_float * nb)(*[float(v) for v in target])
        loss = ctypes.c_double()
        P = (ctypes.c_float * nb)()
        g = torch.empty_like(delta_T) if grad else None
        with self._stream() as stream:
            self._check(self.lib.mx_ps_loss_device(self.ctx, delta_T.data_ptr(), nb, e, t, ctypes.byref(loss), P,
                                                   g.data_ptr() if grad else None, ctypes.c_void_p(stream)))
        return loss.value, list(P), g

    def adjoint(self, snapshot: int, saved, grad_delta_T):
        """Adjoint of ComputeTs + the 21cm box (see mx_adjoint_device) on CUDA
        tensors: (dL/dsfr, dL/dstars, dL/dLXrayGal, dL/dE0)."""
        import torch

        g, device = self._grids(saved)
        if not device:
            raise ValueError("adjoint: device grids only")
        gs = torch.zeros_like(saved["sfr"])
        gst = torch.zeros_like(saved["stars"])
        par = (ctypes.c_double * 2)()
        with self._stream() as stream:
            self._check(self.lib.mx_adjoint_device(self.ctx, snapshot, ctypes.byref(g), grad_delta_T.data_ptr(),
                                                   gs.data_ptr(), gst.data_ptr(), par, ctypes.c_void_p(stream)))
        return gs, gst, par[0], par[1]


class Batch:
    """Native executor of independent boxes (mx_batch_create / mx_batch_run,
    include/mx_reion.h): worker threads with their own contexts and streams,
    kept between runs while a worker's configuration stays the same."""

    def __init__(self, tables_dir: str = TABLES_DIR, max_workers: int = 0, max_work_bytes: int = 0):
        self.lib = _lib.load()
        self.handle = ctypes.c_void_p()
        rc = self.lib.mx_batch_create(tables_dir.encode(), int(max_workers), int(max_work_bytes),
                                      ctypes.byref(self.handle))
        if rc != 0:
            raise _lib.MxError(rc, "mx_batch_create")

    def run(self, items, graph: bool = False):
        """items: dicts with "params" (ReionParams), "redshifts", "snapshot"
        and "grids" (name -> C-contiguous float32 numpy array, updated in place
        as by ReionGridStep.step).  Returns the globals of every item; raises
        MxError if any item failed (the others still ran).  graph=True runs
        every item in one CUDA graph launch (mx_batch_run_graph; the arrays
        must be page-locked, e.g. torch.empty(..., pin_memory=True).numpy())."""
        n = len(items)
        arr = (_lib.MxBatchItem * n)()
        keep = []  # ctypes objects that must outlive the call
        outs = []
        for i, it in enumerate(items):
            pc = it["params"].to_ctypes()
            zz = (ctypes.c_double * len(it["redshifts"]))(*[float(z) for z in it["redshifts"]])
            g = MxGrids()
            for name in GRID_NAMES:
                a = it["grids"].get(name)
                if a is None:
                    continue
                if not isinstance(a, np.ndarray) or a.dtype != np.float32 or not a.flags.c_contiguous:
                    raise ValueError(f"item {i}, {name}: need C-contiguous float32 numpy array")
                setattr(g, name, a.ctypes.data)
            out = MxGlobals()
            keep += [pc, zz, g]
            outs.append(out)
            arr[i].params = ctypes.pointer(pc)
            arr[i].redshifts = zz
            arr[i].n_snaps = len(it["redshifts"])
            arr[i].snapshot = int(it["snapshot"])
            arr[i].grids = ctypes.pointer(g)
            arr[i].out = ctypes.pointer(out)
            arr[i].status = -99
        run = self.lib.mx_batch_run_graph if graph else self.lib.mx_batch_run
        rc = run(self.handle, arr, n)
        if rc != 0:
            raise _lib.MxError(rc, self.lib.mx_batch_last_error(self.handle).decode())
        return [o.as_dict() for o in outs]

    def close(self):
        if self.handle:
            self.lib.mx_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_batch(items, tables_dir: str = TABLES_DIR, max_workers: int = 0, max_work_bytes: int = 0):
    """One-shot Batch(...).run(items)."""
    b = Batch(tables_dir, max_workers, max_work_bytes)
    try:
        return b.run(items)
    finally:
        b.close()
