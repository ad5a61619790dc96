"""ctypes wrapper of liboracle.so (test infrastructure only).

Mirrors the method names of apic_gb300.Apic so a parity test can drive the
GPU library and the CPU oracle through the same calls.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "apic-fluid-simulation_gb300"))
from apic_gb300 import (FIELDS, STAGES, InfoC, RenderParamsC, RenderStatsC, SceneParamsC, StatsC,  # noqa: E402
                        WorldPropsC, WorldProperties)

from . import build as _build  # noqa: E402

_lib = None
_VP = ctypes.c_void_p
_FP = ctypes.POINTER(ctypes.c_float)


def load(rebuild: bool = True) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if rebuild else _build.LIB
    lib = ctypes.CDLL(path)
    sig = {
        "oracle_create": (_VP, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.POINTER(WorldPropsC),
                                ctypes.c_int, ctypes.c_int]),
        "oracle_destroy": (None, [_VP]),
        "oracle_set_threads": (ctypes.c_int, [_VP, ctypes.c_int]),
        "oracle_set_particles": (ctypes.c_int, [_VP, ctypes.c_uint32, _FP, _FP, _FP, _FP]),
        "oracle_set_solver": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_float, ctypes.c_uint32]),
        "oracle_set_warm_start": (ctypes.c_int, [_VP, ctypes.c_int]),
        "oracle_update": (ctypes.c_int, [_VP, ctypes.c_uint32, ctypes.c_float]),
        "oracle_run_stage": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_float]),
        "oracle_finish_substep": (ctypes.c_int, [_VP, ctypes.c_float]),
        "oracle_max_particle_velocity": (ctypes.c_int, [_VP, _FP]),
        "oracle_add_radial_force": (ctypes.c_int, [_VP, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                   ctypes.c_float]),
        "oracle_get_info": (ctypes.c_int, [_VP, ctypes.POINTER(InfoC)]),
        "oracle_get_stats": (ctypes.c_int, [_VP, ctypes.POINTER(StatsC)]),
        "oracle_field_shape": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_uint32)]),
        "oracle_read_field": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_uint64]),
        "oracle_write_field": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_uint64]),
        "oracle_render": (ctypes.c_int, [ctypes.c_uint32, _FP, _FP, _FP, _FP, ctypes.POINTER(RenderParamsC),
                                         ctypes.c_uint32, ctypes.c_float, _VP, ctypes.POINTER(RenderStatsC)]),
        "oracle_morton": (ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_uint32]),
        "oracle_scene_count": (ctypes.c_int, [ctypes.POINTER(SceneParamsC), ctypes.POINTER(ctypes.c_uint64)]),
        "oracle_scene_fill": (ctypes.c_int, [ctypes.POINTER(SceneParamsC), ctypes.c_uint64, _FP, _FP, _FP, _FP]),
        "oracle_random_lane": (ctypes.c_float, [ctypes.c_uint32, ctypes.c_uint32]),
        "oracle_temporal_weight": (ctypes.c_float, [ctypes.c_float]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ck(rc: int, where: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{where} failed with status {rc}")


class OracleSim:
    """CPU restatement of the reference's Apic with the apic_gb300.Apic methods."""

    def __init__(self, width: int, height: int, cell_size: float, props: WorldProperties,
                 fp64: bool = False, threads: int = 1):
        self._lib = load()
        wp = WorldPropsC(props.gravity, props.border_damping, props.cfl, props.solve_error)
        self._h = self._lib.oracle_create(width, height, cell_size, ctypes.byref(wp), 1 if fp64 else 0, threads)
        if not self._h:
            raise RuntimeError("oracle_create failed")
        self.fp64 = fp64

    def close(self) -> None:
        if self._h:
            self._lib.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int) -> None:
        _ck(self._lib.oracle_set_threads(self._h, n), "oracle_set_threads")

    def set_particles(self, px, py, vx=None, vy=None) -> None:
        px = np.ascontiguousarray(px, np.float32)
        py = np.ascontiguousarray(py, np.float32)
        vx = np.zeros_like(px) if vx is None else np.ascontiguousarray(vx, np.float32)
        vy = np.zeros_like(px) if vy is None else np.ascontiguousarray(vy, np.float32)
        f = lambda a: a.ctypes.data_as(_FP)  # noqa: E731
        _ck(self._lib.oracle_set_particles(self._h, len(px), f(px), f(py), f(vx), f(vy)), "oracle_set_particles")

    def set_solver(self, mode: int, rel_tol: float = 1e-6, max_iterations: int = 500) -> None:
        _ck(self._lib.oracle_set_solver(self._h, mode, rel_tol, max_iterations), "oracle_set_solver")

    def set_warm_start(self, enabled: bool) -> None:
        _ck(self._lib.oracle_set_warm_start(self._h, 1 if enabled else 0), "oracle_set_warm_start")

    def update(self, debug_options=None, frame_deltatime: float = 1 / 60) -> None:
        flags = 1 if (debug_options is not None and debug_options.disable_particle_sort) else 0
        _ck(self._lib.oracle_update(self._h, flags, frame_deltatime), "oracle_update")

    def run_stage(self, stage, dt: float) -> None:
        sid = STAGES.index(stage) if isinstance(stage, str) else int(stage)
        _ck(self._lib.oracle_run_stage(self._h, sid, dt), "oracle_run_stage")

    def finish_substep(self, dt: float) -> None:
        _ck(self._lib.oracle_finish_substep(self._h, dt), "oracle_finish_substep")

    def get_max_particle_velocity(self) -> float:
        out = ctypes.c_float(0)
        _ck(self._lib.oracle_max_particle_velocity(self._h, ctypes.byref(out)), "oracle_max_particle_velocity")
        return out.value

    def add_radial_force(self, x: float, y: float, radius: float, strength: float) -> None:
        _ck(self._lib.oracle_add_radial_force(self._h, x, y, radius, strength), "oracle_add_radial_force")

    def info(self) -> InfoC:
        out = InfoC()
        _ck(self._lib.oracle_get_info(self._h, ctypes.byref(out)), "oracle_get_info")
        return out

    def stats(self) -> StatsC:
        out = StatsC()
        _ck(self._lib.oracle_get_stats(self._h, ctypes.byref(out)), "oracle_get_stats")
        return out

    def field_shape(self, fid: int):
        n, e = ctypes.c_uint64(0), ctypes.c_uint32(0)
        _ck(self._lib.oracle_field_shape(self._h, fid, ctypes.byref(n), ctypes.byref(e)), "oracle_field_shape")
        return n.value, e.value

    def _dtype(self, fid: int, e: int):
        if e == 1:
            return np.uint8
        if fid in (48, 49, 52):
            return np.uint32
        if fid in (32, 33, 34, 35) or (fid >= 64 and fid % 256 == 64):
            return np.uint64
        return np.float64 if e == 8 else np.float32

    def read_field(self, field) -> np.ndarray:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        n, e = self.field_shape(fid)
        out = np.zeros(n, self._dtype(fid, e))
        _ck(self._lib.oracle_read_field(self._h, fid, out.ctypes.data, out.nbytes), "oracle_read_field")
        return out

    def write_field(self, field, data: np.ndarray) -> None:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        n, e = self.field_shape(fid)
        data = np.ascontiguousarray(data, self._dtype(fid, e))
        _ck(self._lib.oracle_write_field(self._h, fid, data.ctypes.data, data.nbytes), "oracle_write_field")


def generate_scene(p: SceneParamsC):
    """The scene's particles (pos_x, pos_y, vel_x, vel_y as float32), from the
    same generator as apic_gb300.generate_scene, without the GPU library."""
    lib = load()
    n = ctypes.c_uint64(0)
    _ck(lib.oracle_scene_count(ctypes.byref(p), ctypes.byref(n)), "oracle_scene_count")
    arrs = [np.zeros(n.value, np.float32) for _ in range(4)]
    _ck(lib.oracle_scene_fill(ctypes.byref(p), n.value, *[a.ctypes.data_as(_FP) for a in arrs]), "oracle_scene_fill")
    return tuple(arrs)


def morton(x: int, y: int) -> int:
    return int(load().oracle_morton(x, y))


def random_lane(slot: int, seed: int) -> float:
    return float(load().oracle_random_lane(slot, seed))


def temporal_weight(tau: float) -> float:
    return float(load().oracle_temporal_weight(tau))


def render(px, py, vx, vy, params: RenderParamsC, fluid_cells: int = 0, cell_size: float = 0.0):
    """The oracle's frame (height x width x 4 uint8) and RenderStatsC for the
    particles given as float32 arrays, drawn in index order."""
    lib = load()
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (px, py, vx, vy)]
    n = len(arrs[0])
    frame = np.empty((params.height, params.width, 4), dtype=np.uint8)
    st = RenderStatsC()
    ptr = [a.ctypes.data_as(_FP) for a in arrs]
    _ck(lib.oracle_render(n, *ptr, ctypes.byref(params), fluid_cells, cell_size, frame.ctypes.data_as(_VP),
                          ctypes.byref(st)), "oracle_render")
    return frame, st
