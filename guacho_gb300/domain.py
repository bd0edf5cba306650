"""Host-side mirror of Guacho's hot-path interface over the C ABI.

`Domain` keeps the reference's vocabulary: `boundaryI`, `calcprim`,
`get_timestep`, `tstep` (src/boundaries.f90:44, src/hydro_core.f90:245,623,
src/hydro_solver.f90:134) and the main-loop driver `run`
(src/main.f90:94-125).  Host arrays use the reference's layout: the Fortran
array u(neq, nxmin:nxmax, nymin:nymax, nzmin:nzmax) seen from numpy as a
C-ordered (nz+4, ny+4, nx+4, neq) float64 array.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import check, ptr
from . import params as P
from .params import Params


class Domain:
    """One box on the GPU (device-resident u, up, E, ...)."""

    def __init__(self, params: Params, stream: int | None = None):
        self.params = params
        self._lib = _abi.lib()
        self._ps = _abi.to_struct(params)
        h = C.c_void_p()
        check("gch_create", self._lib.gch_create(C.byref(self._ps), C.c_void_p(stream or 0),
                                                  C.byref(h)))
        self._h = h
        self.time = 0.0
        self.iter = 1          # currentIteration starts at 1 (src/init.f90:125)
        self.tprint = None

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- state transfer -------------------------------------------------
    def upload(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.shape == self.params.shape, (u.shape, self.params.shape)
        check("gch_upload", self._lib.gch_upload(self._h, ptr(u)))

    def download(self, with_primit: bool = False, out: np.ndarray | None = None):
        """u (and primit) in the host layout; `out`, if given, receives u (a
        page-locked `out` is written directly over the host link)."""
        if out is not None:
            assert out.shape == self.params.shape and out.dtype == np.float64
            assert out.flags.c_contiguous
        u = out if out is not None else np.empty(self.params.shape, dtype=np.float64)
        pr = np.empty(self.params.shape, dtype=np.float64) if with_primit else None
        check("gch_download", self._lib.gch_download(self._h, ptr(u),
                                                      ptr(pr) if pr is not None else None))
        return (u, pr) if with_primit else u

    def set_background(self, prim0: np.ndarray) -> None:
        """The background primit0 of SOLVER_HLLE_SPLIT_ALL (layout of u);
        call before init, as the reference's background is part of the
        initial state."""
        prim0 = np.ascontiguousarray(prim0, dtype=np.float64)
        assert prim0.shape == self.params.shape, (prim0.shape, self.params.shape)
        check("gch_set_background", self._lib.gch_set_background(self._h, ptr(prim0)))
        self._prim0 = prim0.copy()  # for the BIN output of the total state

    # ---- reference entry points ----------------------------------------
    def boundaryI(self) -> None:
        check("gch_boundaryI", self._lib.gch_boundaryI(self._h))

    def calcprim(self) -> None:
        check("gch_calcprim", self._lib.gch_calcprim(self._h))

    def get_timestep(self, current_iter: int, n_iter: int, current_time: float,
                     tprint: float) -> tuple[float, bool]:
        dt = C.c_double()
        dump = C.c_int(0)
        check("gch_get_timestep", self._lib.gch_get_timestep(
            self._h, current_iter, n_iter, current_time, tprint, C.byref(dt), C.byref(dump)))
        return dt.value, bool(dump.value)

    def tstep(self, dt: float) -> None:
        check("gch_tstep", self._lib.gch_tstep(self._h, dt))

    def step_host(self, u: np.ndarray, current_iter: int, n_iter: int, current_time: float,
                  tprint: float) -> tuple[float, bool]:
        """get_timestep + tstep with u in host memory (updated in place)."""
        assert u.flags.c_contiguous and u.dtype == np.float64
        dt = C.c_double()
        dump = C.c_int(0)
        check("gch_step_host", self._lib.gch_step_host(
            self._h, ptr(u), current_iter, n_iter, current_time, tprint, C.byref(dt),
            C.byref(dump)))
        return dt.value, bool(dump.value)

    # ---- drivers ----------------------------------------------------------
    def init(self, u0: np.ndarray) -> None:
        """src/main.f90:73-79: initial state, boundaryI, calcprim."""
        self.upload(u0)
        self.boundaryI()
        self.calcprim()

    def run(self, tmax: float, dtprint: float, max_steps: int = 1 << 20, n_iter: int = 10,
            device_loop: bool = True) -> int:
        """The time loop of src/main.f90:94-125 (without output)."""
        if self.tprint is None:
            self.tprint = dtprint
        if device_loop:
            t = C.c_double(self.time)
            it = C.c_int(self.iter)
            tp = C.c_double(self.tprint)
            done = C.c_int(0)
            check("gch_advance", self._lib.gch_advance(
                self._h, max_steps, tmax, dtprint, n_iter, C.byref(t), C.byref(it),
                C.byref(tp), C.byref(done)))
            self.time, self.iter, self.tprint = t.value, it.value, tp.value
            return done.value
        steps = 0
        while self.time <= tmax and steps < max_steps:
            dt, dump = self.get_timestep(self.iter, n_iter, self.time, self.tprint)
            self.tstep(dt)
            self.time = self.time + dt
            if dump:
                self.tprint = self.tprint + dtprint
            self.iter += 1
            steps += 1
        return steps

    def write_output(self, outputpath, itprint: int, dump_divb: bool = True,
                     scal=(1.0, 1.0, 1.0)) -> None:
        """src/output.f90:40-53 write_output with out_bin: download u and
        write BIN/points000.<itprint>.bin (+ the div B dump when MHD)."""
        from . import binio
        u = self.download()
        split = self.params.riemann_solver == P.SOLVER_HLLE_SPLIT_ALL
        prim0 = getattr(self, "_prim0", np.zeros(self.params.shape)) if split else None
        binio.write_bin(binio.bin_path(outputpath, itprint), u, self.params, scal, prim0=prim0)
        if dump_divb and self.params.bfield:
            binio.write_divb(binio.bin_path(outputpath, itprint, base="divB-"), u,
                             self.params, scal)

    def read_warm_start(self, path) -> None:
        """src/init.f90:437-467 (iwarm): read u from a BIN file, then
        calcprim."""
        from . import binio
        hdr, u = binio.read_bin(path)
        if (hdr["nx"], hdr["ny"], hdr["nz"], hdr["neq"]) != (
                self.params.nx, self.params.ny, self.params.nz, self.params.neq):
            raise ValueError(f"{path}: grid {hdr} does not match the domain")
        self.upload(u)
        self.calcprim()

    def step_info(self) -> tuple[int, int]:
        pf = C.c_longlong()
        err = C.c_int()
        check("gch_last_step_info", self._lib.gch_last_step_info(self._h, C.byref(pf),
                                                                  C.byref(err)))
        return pf.value, err.value

    def tc_info(self) -> tuple[int, float]:
        """Conduction substeps of the last tstep and the conduction
        timescale in seconds (src/thermal_cond.f90:690-733)."""
        n = C.c_int()
        dtc = C.c_double()
        check("gch_tc_info", self._lib.gch_tc_info(self._h, C.byref(n), C.byref(dtc)))
        return n.value, dtc.value

    def launches_per_step(self) -> int:
        return self._lib.gch_launches_per_step(self._h)

    def step_host_overlaps(self) -> bool:
        """Whether step_host copies u back behind the second half step."""
        return bool(self._lib.gch_step_host_overlaps(self._h))

    @property
    def kz(self) -> int:
        """z planes per block of the stage kernels."""
        return self._lib.gch_get_kz(self._h)

    @kz.setter
    def kz(self, value: int) -> None:
        check("gch_set_kz", self._lib.gch_set_kz(self._h, int(value)))

    def autotune(self) -> dict:
        """Time the stage-1 kernel for each candidate depth on the current
        state, keep the fastest; returns {kz: ms}."""
        ck = (C.c_int * 16)()
        cm = (C.c_float * 16)()
        n = C.c_int()
        check("gch_autotune", self._lib.gch_autotune(self._h, 16, ck, cm, C.byref(n)))
        return {int(ck[i]): float(cm[i]) for i in range(n.value)}

    def advance_timed(self, steps: int, n_iter: int = 10) -> float:
        """`steps` device-resident steps timed with CUDA events; GPU ms."""
        ms = C.c_float()
        check("gch_advance_timed", self._lib.gch_advance_timed(self._h, steps, n_iter,
                                                                C.byref(ms)))
        return ms.value

    def profile_step(self) -> list[tuple[str, float]]:
        """One step with an event after every launch: [(kernel, ms)]."""
        cap, nl = 64, 32
        ms = (C.c_float * cap)()
        names = C.create_string_buffer(cap * nl)
        n = C.c_int()
        check("gch_profile_step", self._lib.gch_profile_step(self._h, cap, ms, names, nl,
                                                              C.byref(n)))
        raw = names.raw
        return [(raw[i * nl:(i + 1) * nl].split(b"\0")[0].decode(), ms[i])
                for i in range(n.value)]


class Batch:
    """Independent boxes of uneven size, each with its own CFL dt."""

    def __init__(self, params_list: list[Params]):
        self.params = list(params_list)
        self._lib = _abi.lib()
        arr = (_abi.Params_t * len(self.params))(*[_abi.to_struct(p) for p in self.params])
        self._arr = arr
        h = C.c_void_p()
        check("gch_batch_create", self._lib.gch_batch_create(len(self.params), arr, None,
                                                              C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gch_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, box: int, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, dtype=np.float64)
        check("gch_batch_upload", self._lib.gch_batch_upload(self._h, box, ptr(u)))

    def download(self, box: int) -> np.ndarray:
        u = np.empty(self.params[box].shape, dtype=np.float64)
        check("gch_batch_download", self._lib.gch_batch_download(self._h, box, ptr(u)))
        return u

    def advance(self, steps: int, n_iter: int = 10) -> None:
        check("gch_batch_advance", self._lib.gch_batch_advance(self._h, steps, n_iter))

    def times(self):
        n = len(self.params)
        t = (C.c_double * n)()
        it = (C.c_int * n)()
        check("gch_batch_time", self._lib.gch_batch_time(self._h, t, it))
        return list(t), list(it)

    def tuning(self) -> dict:
        """Grouped mode, the z-march depth and launch form chosen by the
        autotuner (blocks_per_sm: resident blocks per SM of the persistent
        stage kernels, 0 for one block per work item), and the measured
        stage-1 time of every candidate pair ({(kz, blocks_per_sm): ms});
        kz-only candidates at the chosen launch form under "candidates"."""
        g, kz, bps, n = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        cap = 64
        ck, cb = (C.c_int * cap)(), (C.c_int * cap)()
        cm = (C.c_float * cap)()
        check("gch_batch_tuning_grid", self._lib.gch_batch_tuning_grid(
            self._h, C.byref(g), C.byref(kz), C.byref(bps), cap, ck, cb, cm, C.byref(n)))
        grid = {(int(ck[i]), int(cb[i])): float(cm[i]) for i in range(n.value)}
        return {"grouped": bool(g.value), "kz": kz.value, "blocks_per_sm": bps.value,
                "candidates": {k: v for (k, b), v in grid.items() if b == bps.value},
                "grid": grid}
