"""GB300 APIC/FLIP step behind the reference's simulation API.

Python mirror of the reference crate's public interface (src/apic.rs):
``WorldProperties`` (:707-713), ``DebugOptions`` (:397-400) and ``Apic`` with
``new`` (:779), ``update`` (:2429), ``add_radial_force`` (:2352),
``get_max_particle_velocity`` (:2412), ``is_fluid`` (:1015) and accessors for
the public fields that src/main.rs reads.  Every call goes through the C-ABI
of ``libapic_gpu.so`` (include/apic_gpu.h); there is no CPU fallback: loading
fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG_ROOT, "lib", "libapic_gpu.so")

# ---- constants (include/apic_gpu.h) ---------------------------------------
OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_NONFINITE, ERR_NOT_CONVERGED, ERR_NO_DEVICE = range(8)
ERR_UNSUPPORTED = 8
UPDATE_DISABLE_SORT = 0x1
UPDATE_BATCH_STREAMS = 0x2  # apic_update_batch: each scene on its own stream
UPDATE_BATCH_JOINT = 0x4    # apic_update_batch: the joint form whenever it applies
SOLVER_REFERENCE, SOLVER_REL_FP32, SOLVER_REL_MIXED = 0, 1, 2
SERVER_ROUNDS, SERVER_CONTINUOUS = 0, 1
SCENE_REFERENCE_DEFAULT, SCENE_DAM_BREAK, SCENE_DAM_BREAK_DISK, SCENE_NOISE = 0, 1, 2, 3
OPT_PDL = 4
OPT_DSM_VCYCLE = 5
OPT_WARM_START = 7
OPT_STREAM_PRIORITY = 8
OPT_P2G_ORDER = 9  # 0 follow the solver mode, 1 the reference's order, 2 cell order

FIELDS = {
    "pos_x": 0, "pos_y": 1, "vel_x": 2, "vel_y": 3, "cu_x": 4, "cu_y": 5, "cv_x": 6, "cv_y": 7, "tres": 8,
    "u": 16, "v": 17, "valid_u": 18, "valid_v": 19,
    "density": 24, "smoothed_density": 25, "pressure": 26,
    "fluid_bits": 32, "obstacle_bits": 33, "u_open_bits": 34, "v_open_bits": 35,
    "residual": 40, "diag": 41, "inv_diag": 42, "plus_x": 43, "plus_y": 44, "error": 45,
    "sort_keys": 48, "sort_vals": 49, "fluid_list": 52,
    "ext_force_u": 56, "ext_force_v": 57, "post_force_u": 58, "post_force_v": 59,
}
MG_FIELDS = {"fluid_bits": 64, "diag": 65, "inv_diag": 66, "plus_x": 67, "plus_y": 68}
MG_LEVEL_STRIDE = 256
STAGES = ["sort", "p2g", "forces", "build", "mg", "pcg", "grad", "post", "extrap", "g2p", "vmax", "vcycle"]
PARTICLE_FIELDS = ["pos_x", "pos_y", "vel_x", "vel_y", "cu_x", "cu_y", "cv_x", "cv_y", "tres"]


def mg_field(name: str, level: int) -> int:
    return MG_FIELDS[name] + MG_LEVEL_STRIDE * level


class WorldPropsC(ctypes.Structure):
    _fields_ = [("gravity", ctypes.c_float), ("border_damping", ctypes.c_float),
                ("cfl", ctypes.c_float), ("solve_error", ctypes.c_float)]


class InfoC(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("cells", ctypes.c_uint32),
                ("cell_size", ctypes.c_float), ("num_chunks", ctypes.c_uint32),
                ("num_particles", ctypes.c_uint32), ("fluid_cells", ctypes.c_uint32),
                ("timestamp", ctypes.c_uint32), ("prev_deltatime", ctypes.c_float),
                ("mg_levels", ctypes.c_uint32)]


class StatsC(ctypes.Structure):
    _fields_ = [("substeps", ctypes.c_uint32), ("pcg_iterations", ctypes.c_uint32),
                ("pcg_iterations_total", ctypes.c_uint32), ("refinement_steps", ctypes.c_uint32),
                ("residual_max", ctypes.c_float), ("residual_rel", ctypes.c_float),
                ("true_residual_rel", ctypes.c_double), ("not_converged", ctypes.c_uint32),
                ("nonfinite_lanes", ctypes.c_uint32), ("kernel_launches", ctypes.c_uint64),
                ("solve_ms", ctypes.c_double)]


class SceneParamsC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("cell_size", ctypes.c_float), ("sub", ctypes.c_uint32), ("seed", ctypes.c_uint32),
                ("fluid_x", ctypes.c_float), ("fluid_y", ctypes.c_float),
                ("disk_x", ctypes.c_float), ("disk_y", ctypes.c_float), ("disk_r", ctypes.c_float),
                ("disk_vx", ctypes.c_float), ("disk_vy", ctypes.c_float),
                ("noise_period", ctypes.c_float), ("noise_threshold", ctypes.c_float),
                ("vel_sigma", ctypes.c_float)]


class ServerRoundC(ctypes.Structure):
    _fields_ = [("admitted", ctypes.c_uint32), ("stepped", ctypes.c_uint32), ("completed", ctypes.c_uint32),
                ("active", ctypes.c_uint32), ("queued", ctypes.c_uint32), ("round_ms", ctypes.c_double),
                ("memory_used", ctypes.c_uint64)]


class RequestInfoC(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("finished", ctypes.c_uint32), ("steps_done", ctypes.c_uint32),
                ("particles", ctypes.c_uint64), ("substeps", ctypes.c_uint64), ("pcg_iterations", ctypes.c_uint64),
                ("max_true_residual", ctypes.c_double), ("submit_ms", ctypes.c_double),
                ("admit_ms", ctypes.c_double), ("done_ms", ctypes.c_double), ("bytes", ctypes.c_uint64),
                ("result_floats", ctypes.c_uint64)]


class BatchInfoC(ctypes.Structure):
    _fields_ = [("scenes", ctypes.c_uint32), ("joint", ctypes.c_uint32), ("batch_kernel_launches", ctypes.c_uint64),
                ("substep_rounds", ctypes.c_uint32), ("refine_rounds", ctypes.c_uint32),
                ("pcg_rounds", ctypes.c_uint32), ("tuned", ctypes.c_uint32), ("chunk_segs", ctypes.c_uint32),
                ("block_group", ctypes.c_uint32)]


class ServerStatsC(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("active", ctypes.c_uint64), ("queued", ctypes.c_uint64), ("rounds", ctypes.c_uint64),
                ("particle_substeps", ctypes.c_uint64), ("particle_updates", ctypes.c_uint64),
                ("busy_ms", ctypes.c_double), ("elapsed_ms", ctypes.c_double),
                ("step_p50_ms", ctypes.c_double), ("step_p99_ms", ctypes.c_double),
                ("request_p50_ms", ctypes.c_double), ("request_p99_ms", ctypes.c_double),
                ("memory_used", ctypes.c_uint64), ("memory_peak", ctypes.c_uint64),
                ("updates", ctypes.c_uint64), ("prepare_ms", ctypes.c_double), ("host_ms", ctypes.c_double),
                ("mode", ctypes.c_int32), ("prepare_threads", ctypes.c_uint32),
                ("kernel_launches", ctypes.c_uint64)]


class RenderParamsC(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("scale", ctypes.c_float),
                ("draw_radius", ctypes.c_float), ("margin", ctypes.c_float), ("pick_x", ctypes.c_float),
                ("pick_y", ctypes.c_float), ("pick_radius", ctypes.c_float), ("background", ctypes.c_uint32)]


class RenderStatsC(ctypes.Structure):
    _fields_ = [("valid", ctypes.c_uint32), ("nan", ctypes.c_uint32), ("out_of_bounds", ctypes.c_uint32),
                ("fluid_cells", ctypes.c_uint32), ("picked", ctypes.c_int64), ("volume", ctypes.c_float),
                ("kernels", ctypes.c_uint32)]


def render_params(width: int = 1920, height: int = 1080, scale: float | None = None, grid_width: int = 256,
                  cell_size: float = 0.075, draw_radius: float = 3.0, margin: float = 50.0, pick=None,
                  pick_radius: float = 12.0, background=(0, 0, 0)) -> RenderParamsC:
    """Parameters of the GUI's particle view (src/main.rs:26-36): a 1920 x 1080
    frame, SIM_SCALE = WIDTH / (GRID_WIDTH * CELL_SIZE) pixels per unit unless
    `scale` is given, 3-pixel discs, a 50-pixel out-of-bounds margin; `pick`:
    (x, y) in pixels to pick the nearest particle within `pick_radius`."""
    if scale is None:
        scale = float(np.float32(width) / (np.float32(grid_width) * np.float32(cell_size)))
    px, py, pr = (0.0, 0.0, -1.0) if pick is None else (float(pick[0]), float(pick[1]), float(pick_radius))
    r, g, b = background
    return RenderParamsC(width, height, scale, draw_radius, margin, px, py, pr,
                         (int(r) & 255) | ((int(g) & 255) << 8) | ((int(b) & 255) << 16) | (255 << 24))


# Every symbol that include/apic_gpu.h declares, with its ctypes signature.
_VP = ctypes.c_void_p
_FP = ctypes.POINTER(ctypes.c_float)
SIGNATURES = {
    "apic_scene_count": (ctypes.c_int, [ctypes.POINTER(SceneParamsC), ctypes.POINTER(ctypes.c_uint64)]),
    "apic_scene_fill": (ctypes.c_int, [ctypes.POINTER(SceneParamsC), ctypes.c_uint64, _FP, _FP, _FP, _FP]),
    "apic_create": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                   ctypes.POINTER(WorldPropsC), ctypes.POINTER(_VP)]),
    "apic_destroy": (ctypes.c_int, [_VP]),
    "apic_last_error": (ctypes.c_char_p, []),
    "apic_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "apic_update": (ctypes.c_int, [_VP, ctypes.c_uint32, ctypes.c_float]),
    "apic_add_radial_force": (ctypes.c_int, [_VP, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "apic_max_particle_velocity": (ctypes.c_int, [_VP, _FP]),
    "apic_is_fluid": (ctypes.c_int, [_VP, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)]),
    "apic_update_world": (ctypes.c_int, [_VP]),
    "apic_get_info": (ctypes.c_int, [_VP, ctypes.POINTER(InfoC)]),
    "apic_get_stats": (ctypes.c_int, [_VP, ctypes.POINTER(StatsC)]),
    "apic_field_shape": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                        ctypes.POINTER(ctypes.c_uint32)]),
    "apic_read_field": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_uint64]),
    "apic_write_field": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_uint64]),
    "apic_read_vec2x8": (ctypes.c_int, [_VP, ctypes.c_int, _FP, ctypes.c_uint64]),
    "apic_update_async": (ctypes.c_int, [_VP, ctypes.c_uint32, ctypes.c_float]),
    "apic_update_wait": (ctypes.c_int, [_VP]),
    "apic_stage_field": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_uint64]),
    "apic_read_vec2x8_async": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_uint64]),
    "apic_read_wait": (ctypes.c_int, [_VP]),
    "apic_set_particles": (ctypes.c_int, [_VP, ctypes.c_uint32, _FP, _FP, _FP, _FP]),
    "apic_set_solver": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_float, ctypes.c_uint32]),
    "apic_set_profiling": (ctypes.c_int, [_VP, ctypes.c_int]),
    "apic_set_option": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int]),
    "apic_get_option": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "apic_get_stage_times": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]),
    "apic_reset_stage_times": (ctypes.c_int, [_VP]),
    "apic_synchronize": (ctypes.c_int, [_VP]),
    "apic_get_stream": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "apic_debug_run_stage": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_float]),
    "apic_morton_sort_noalloc": (ctypes.c_int, [_VP, _VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                ctypes.c_float, _VP, _VP, _VP]),
    "apic_debug_finish_substep": (ctypes.c_int, [_VP, ctypes.c_float]),
    "apic_update_batch": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                         ctypes.POINTER(ctypes.c_int)]),
    "apic_batch_last_info": (ctypes.c_int, [ctypes.POINTER(BatchInfoC)]),
    "apic_place_scenes": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                         ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32,
                                         ctypes.POINTER(ctypes.c_int32)]),
    "apic_scene_bytes": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "apic_server_create": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_VP)]),
    "apic_server_destroy": (ctypes.c_int, [_VP]),
    "apic_server_set_mode": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_uint32]),
    "apic_server_scene_option": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]),
    "apic_server_set_work_limit": (ctypes.c_int, [_VP, ctypes.c_uint64]),
    "apic_server_submit": (ctypes.c_int, [_VP, ctypes.POINTER(SceneParamsC), ctypes.POINTER(WorldPropsC),
                                          ctypes.c_uint32, ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]),
    "apic_server_step": (ctypes.c_int, [_VP, ctypes.POINTER(ServerRoundC)]),
    "apic_server_request": (ctypes.c_int, [_VP, ctypes.c_uint64, ctypes.POINTER(RequestInfoC)]),
    "apic_server_result_positions": (ctypes.c_int, [_VP, ctypes.c_uint64, _FP, ctypes.c_uint64]),
    "apic_server_get_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ServerStatsC)]),
    "apic_snapshot_bytes": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_uint64)]),
    "apic_snapshot": (ctypes.c_int, [_VP, _VP, ctypes.c_uint64]),
    "apic_restore": (ctypes.c_int, [_VP, _VP, ctypes.c_uint64]),
    "apic_render": (ctypes.c_int, [_VP, ctypes.POINTER(RenderParamsC), ctypes.POINTER(RenderStatsC)]),
    "apic_read_frame": (ctypes.c_int, [_VP, _VP, ctypes.c_uint64]),
    "apic_frame_device_ptr": (ctypes.c_int, [_VP, ctypes.POINTER(_VP), ctypes.POINTER(ctypes.c_uint32),
                                             ctypes.POINTER(ctypes.c_uint32)]),
}

_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libapic_gpu.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libapic_gpu.so not built ({path}); run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class ApicError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = load_library().apic_last_error().decode(errors="replace")
        super().__init__(f"{where} failed with status {code}: {msg}")
        self.code = code


def _check(code: int, where: str) -> None:
    if code != OK:
        raise ApicError(code, where)


def device_count() -> int:
    n = ctypes.c_int(0)
    _check(load_library().apic_device_count(ctypes.byref(n)), "apic_device_count")
    return n.value


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_FP)


# ---- scenes ---------------------------------------------------------------
def scene_params(kind: int, width: int, height: int | None = None, cell_size: float = 0.0, sub: int = 2,
                 seed: int = 0, fluid_x: float = 0.0, fluid_y: float = 0.0, disk=(0.0, 0.0, 0.0),
                 disk_v=(0.0, 0.0), noise_period: float = 0.05, noise_threshold: float = 0.5,
                 vel_sigma: float = 0.0) -> SceneParamsC:
    height = width if height is None else height
    return SceneParamsC(kind, width, height, cell_size, sub, seed, fluid_x, fluid_y, disk[0], disk[1], disk[2],
                        disk_v[0], disk_v[1], noise_period, noise_threshold, vel_sigma)


def scene_count(p: SceneParamsC) -> int:
    """Number of particles the scene holds (apic_scene_count; host code only)."""
    n = ctypes.c_uint64(0)
    _check(load_library().apic_scene_count(ctypes.byref(p), ctypes.byref(n)), "apic_scene_count")
    return n.value


def generate_scene(p: SceneParamsC):
    """Particles of a scene as float32 arrays (pos_x, pos_y, vel_x, vel_y)."""
    lib = load_library()
    n = ctypes.c_uint64(0)
    _check(lib.apic_scene_count(ctypes.byref(p), ctypes.byref(n)), "apic_scene_count")
    arrs = [np.zeros(n.value, np.float32) for _ in range(4)]
    _check(lib.apic_scene_fill(ctypes.byref(p), n.value, *[_fptr(a) for a in arrs]), "apic_scene_fill")
    return tuple(arrs)


# ---- the reference's API ---------------------------------------------------
@dataclass
class WorldProperties:  # src/apic.rs:707-713
    gravity: float = -9.81
    border_damping: float = 0.1
    cfl: float = 5.0
    solve_error: float = 1e-5


@dataclass
class DebugOptions:  # src/apic.rs:397-400
    disable_particle_sort: bool = False


class Apic:
    """Drop-in for the reference's ``Apic`` (src/apic.rs:716-776), state on the GPU."""

    def __init__(self, width: int, height: int, cell_size: float, world_properties: WorldProperties):
        lib = load_library()
        self._lib = lib
        self.world_properties = world_properties
        wp = WorldPropsC(world_properties.gravity, world_properties.border_damping, world_properties.cfl,
                         world_properties.solve_error)
        h = _VP()
        _check(lib.apic_create(width, height, cell_size, ctypes.byref(wp), ctypes.byref(h)), "apic_create")
        self._h = h

    @classmethod
    def new(cls, width: int, height: int, cell_size: float, world_properties: WorldProperties) -> "Apic":
        return cls(width, height, cell_size, world_properties)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.apic_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- step and interaction
    def update(self, debug_options: DebugOptions, frame_deltatime: float) -> None:
        flags = UPDATE_DISABLE_SORT if debug_options.disable_particle_sort else 0
        _check(self._lib.apic_update(self._h, flags, frame_deltatime), "apic_update")

    # pipelined host I/O (stream-ordered; host buffers given by address and
    # size, pinned for the copies to overlap)
    def update_async(self, debug_options: DebugOptions, frame_deltatime: float) -> None:
        flags = UPDATE_DISABLE_SORT if debug_options.disable_particle_sort else 0
        _check(self._lib.apic_update_async(self._h, flags, frame_deltatime), "apic_update_async")

    def update_wait(self) -> None:
        _check(self._lib.apic_update_wait(self._h), "apic_update_wait")

    def stage_field(self, field, host_ptr: int, nbytes: int) -> None:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        _check(self._lib.apic_stage_field(self._h, fid, ctypes.c_void_p(host_ptr), nbytes), "apic_stage_field")

    def read_vec2x8_async(self, which: int, host_ptr: int, nfloats: int) -> None:
        _check(self._lib.apic_read_vec2x8_async(self._h, which, ctypes.c_void_p(host_ptr), nfloats),
               "apic_read_vec2x8_async")

    def read_wait(self) -> None:
        _check(self._lib.apic_read_wait(self._h), "apic_read_wait")

    def add_radial_force(self, world_x: float, world_y: float, radius: float, strength: float) -> None:
        _check(self._lib.apic_add_radial_force(self._h, world_x, world_y, radius, strength), "apic_add_radial_force")

    def get_max_particle_velocity(self) -> float:
        out = ctypes.c_float(0)
        _check(self._lib.apic_max_particle_velocity(self._h, ctypes.byref(out)), "apic_max_particle_velocity")
        return out.value

    def is_fluid(self, i: int, j: int) -> int:
        out = ctypes.c_uint64(0)
        _check(self._lib.apic_is_fluid(self._h, i, j, ctypes.byref(out)), "apic_is_fluid")
        return out.value

    def update_world(self) -> None:
        _check(self._lib.apic_update_world(self._h), "apic_update_world")

    # -- configuration
    def set_particles(self, px, py, vx=None, vy=None) -> None:
        px = np.ascontiguousarray(px, np.float32)
        py = np.ascontiguousarray(py, np.float32)
        vx = np.zeros_like(px) if vx is None else np.ascontiguousarray(vx, np.float32)
        vy = np.zeros_like(px) if vy is None else np.ascontiguousarray(vy, np.float32)
        _check(self._lib.apic_set_particles(self._h, len(px), _fptr(px), _fptr(py), _fptr(vx), _fptr(vy)),
               "apic_set_particles")

    def set_solver(self, mode: int, rel_tol: float = 1e-6, max_iterations: int = 500) -> None:
        _check(self._lib.apic_set_solver(self._h, mode, rel_tol, max_iterations), "apic_set_solver")

    # -- state
    def info(self) -> InfoC:
        out = InfoC()
        _check(self._lib.apic_get_info(self._h, ctypes.byref(out)), "apic_get_info")
        return out

    def stats(self) -> StatsC:
        out = StatsC()
        _check(self._lib.apic_get_stats(self._h, ctypes.byref(out)), "apic_get_stats")
        return out

    @property
    def num_particles(self) -> int:
        return self.info().num_particles

    @property
    def num_chunks(self) -> int:
        return self.info().num_chunks

    @property
    def width(self) -> int:
        return self.info().width

    @property
    def height(self) -> int:
        return self.info().height

    @property
    def cell_size(self) -> float:
        return self.info().cell_size

    @property
    def timestamp(self) -> int:
        return self.info().timestamp

    @property
    def prev_deltatime(self) -> float:
        return self.info().prev_deltatime

    def field_shape(self, field: int):
        n, e = ctypes.c_uint64(0), ctypes.c_uint32(0)
        _check(self._lib.apic_field_shape(self._h, field, ctypes.byref(n), ctypes.byref(e)), "apic_field_shape")
        return n.value, e.value

    def read_field(self, field) -> np.ndarray:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        n, e = self.field_shape(fid)
        dtype = {1: np.uint8, 4: (np.uint32 if fid in (48, 49, 52) else np.float32), 8: np.uint64}[e]
        out = np.zeros(n, dtype)
        _check(self._lib.apic_read_field(self._h, fid, out.ctypes.data, out.nbytes), "apic_read_field")
        return out

    def write_field(self, field, data: np.ndarray) -> None:
        fid = FIELDS[field] if isinstance(field, str) else int(field)
        data = np.ascontiguousarray(data)
        _check(self._lib.apic_write_field(self._h, fid, data.ctypes.data, data.nbytes), "apic_write_field")

    def read_vec2x8(self, which: int) -> np.ndarray:
        """Particle pair field in the reference's Vec2x8 layout: (num_chunks, 2, 8)."""
        nc = self.num_chunks
        out = np.zeros((nc, 2, 8), np.float32)
        _check(self._lib.apic_read_vec2x8(self._h, which, _fptr(out), out.size), "apic_read_vec2x8")
        return out

    @property
    def part_positions(self) -> np.ndarray:
        return self.read_vec2x8(0)

    @property
    def part_velocities(self) -> np.ndarray:
        return self.read_vec2x8(1)

    @property
    def part_c_u(self) -> np.ndarray:
        return self.read_vec2x8(2)

    @property
    def part_c_v(self) -> np.ndarray:
        return self.read_vec2x8(3)

    @property
    def part_time_residual(self) -> np.ndarray:
        return self.read_field("tres").reshape(-1, 8)

    @property
    def mac_pressure_grid(self) -> np.ndarray:
        return self.read_field("pressure")

    @property
    def mac_density(self) -> np.ndarray:
        return self.read_field("density")

    @property
    def smoothed_density(self) -> np.ndarray:
        return self.read_field("smoothed_density")

    def set_option(self, option: int, value: int) -> None:
        _check(self._lib.apic_set_option(self._h, option, value), "apic_set_option")

    def get_option(self, option: int) -> int:
        v = ctypes.c_int(0)
        _check(self._lib.apic_get_option(self._h, option, ctypes.byref(v)), "apic_get_option")
        return v.value

    # -- snapshot / restore (the state a later update reads)
    def snapshot(self) -> bytes:
        n = ctypes.c_uint64()
        _check(self._lib.apic_snapshot_bytes(self._h, ctypes.byref(n)), "apic_snapshot_bytes")
        buf = ctypes.create_string_buffer(n.value)
        _check(self._lib.apic_snapshot(self._h, ctypes.cast(buf, _VP), n.value), "apic_snapshot")
        return buf.raw

    def restore(self, blob: bytes) -> None:
        buf = ctypes.create_string_buffer(bytes(blob), len(blob))
        _check(self._lib.apic_restore(self._h, ctypes.cast(buf, _VP), len(blob)), "apic_restore")

    # -- headless particle view (src/main.rs:207-277)
    def render(self, params: RenderParamsC | None = None, read: bool = True):
        """Splat the particles into the scene's device frame; returns (frame as
        a height x width x 4 uint8 array, or None when read is False; stats)."""
        p = params if params is not None else render_params()
        st = RenderStatsC()
        _check(self._lib.apic_render(self._h, ctypes.byref(p), ctypes.byref(st)), "apic_render")
        if not read:
            return None, st
        frame = np.empty((p.height, p.width, 4), dtype=np.uint8)
        _check(self._lib.apic_read_frame(self._h, frame.ctypes.data_as(_VP), frame.nbytes), "apic_read_frame")
        return frame, st

    def frame_device_ptr(self):
        ptr, w, h = _VP(), ctypes.c_uint32(), ctypes.c_uint32()
        _check(self._lib.apic_frame_device_ptr(self._h, ctypes.byref(ptr), ctypes.byref(w), ctypes.byref(h)),
               "apic_frame_device_ptr")
        return ptr.value, w.value, h.value

    # -- measurement and testing hooks
    def set_profiling(self, on: bool) -> None:
        _check(self._lib.apic_set_profiling(self._h, 1 if on else 0), "apic_set_profiling")

    def stage_times(self):
        n = len(STAGES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_uint64 * n)()
        _check(self._lib.apic_get_stage_times(self._h, ms, cnt, n), "apic_get_stage_times")
        return {STAGES[i]: (ms[i], cnt[i]) for i in range(n)}

    def reset_stage_times(self) -> None:
        _check(self._lib.apic_reset_stage_times(self._h), "apic_reset_stage_times")

    def synchronize(self) -> None:
        _check(self._lib.apic_synchronize(self._h), "apic_synchronize")

    def run_stage(self, stage, dt: float) -> None:
        sid = STAGES.index(stage) if isinstance(stage, str) else int(stage)
        _check(self._lib.apic_debug_run_stage(self._h, sid, dt), "apic_debug_run_stage")

    def finish_substep(self, dt: float) -> None:
        _check(self._lib.apic_debug_finish_substep(self._h, dt), "apic_debug_finish_substep")


# ---- batched and served scenes (no counterpart in the reference) -------------

def update_batch(sims, debug_options: DebugOptions | None = None, frame_deltatime: float = 1 / 60,
                 streams: bool = False, joint: bool = False) -> list[int]:
    """One update of every scene in `sims` (apic_update_batch), in the form
    the library's batch tuner chose for this makeup of scenes: the pressure
    solves as one launch per phase over all scenes, or every scene's update
    on its own stream.  streams=True / joint=True force one of the two."""
    lib = load_library()
    flags = UPDATE_DISABLE_SORT if (debug_options is not None and debug_options.disable_particle_sort) else 0
    if streams:
        flags |= UPDATE_BATCH_STREAMS
    if joint:
        flags |= UPDATE_BATCH_JOINT
    arr = (_VP * len(sims))(*[s._h for s in sims])
    status = (ctypes.c_int * len(sims))()
    _check(lib.apic_update_batch(arr, len(sims), flags, frame_deltatime, status), "apic_update_batch")
    return list(status)


def batch_last_info() -> dict:
    """The last update_batch call: scenes, joint (1: solves as one launch per
    phase), the batch's own kernel launches and its loop rounds."""
    out = BatchInfoC()
    _check(load_library().apic_batch_last_info(ctypes.byref(out)), "apic_batch_last_info")
    return {f: getattr(out, f) for f, _ in BatchInfoC._fields_}


def scene_bytes(width: int, height: int, particles: int) -> int:
    out = ctypes.c_uint64(0)
    _check(load_library().apic_scene_bytes(width, height, particles, ctypes.byref(out)), "apic_scene_bytes")
    return out.value


def place_scenes(bytes_per_scene, work_per_scene, budgets):
    """Device of each independent scene on len(budgets) GPUs (apic_place_scenes):
    largest scenes first, each to the least-loaded device whose memory budget
    still holds it; -1 where none does.  The same on every rank."""
    n, d = len(bytes_per_scene), len(budgets)
    b = (ctypes.c_uint64 * max(n, 1))(*[int(x) for x in bytes_per_scene])
    w = (ctypes.c_uint64 * max(n, 1))(*[int(x) for x in work_per_scene])
    bud = (ctypes.c_uint64 * max(d, 1))(*[int(x) for x in budgets])
    out = (ctypes.c_int32 * max(n, 1))()
    _check(load_library().apic_place_scenes(b, w, n, bud, d, out), "apic_place_scenes")
    return [int(out[i]) for i in range(n)]


class Server:
    """Continuous-batching request loop over independent scenes (apic_server_*)."""

    def __init__(self, memory_budget_bytes: int, max_active: int, keep_results: bool = False,
                 mode: int = None, prepare_threads: int = 4):
        self._lib = load_library()
        h = _VP()
        _check(self._lib.apic_server_create(memory_budget_bytes, max_active, 1 if keep_results else 0,
                                            ctypes.byref(h)), "apic_server_create")
        self._h = h
        if mode is not None:
            self.set_mode(mode, prepare_threads)

    def set_mode(self, mode: int, prepare_threads: int = 4) -> None:
        """SERVER_CONTINUOUS (default) or SERVER_ROUNDS; only while no scene is admitted."""
        _check(self._lib.apic_server_set_mode(self._h, mode, prepare_threads), "apic_server_set_mode")

    def set_work_limit(self, max_active_cells: int) -> None:
        """Admit while the admitted scenes' grid cells stay within max_active_cells (0: no limit)."""
        _check(self._lib.apic_server_set_work_limit(self._h, max_active_cells), "apic_server_set_work_limit")

    def scene_option(self, option: int, value: int, min_cells: int = 0, max_cells: int = (1 << 64) - 1) -> None:
        """Apic.set_option(option, value) on every scene with min_cells..max_cells cells."""
        _check(self._lib.apic_server_scene_option(self._h, option, value, min_cells, max_cells),
               "apic_server_scene_option")

    def submit(self, scene: SceneParamsC, props: WorldProperties, steps: int, frame_deltatime: float,
               solver: int = SOLVER_REL_MIXED, rel_tol: float = 1e-6, max_iterations: int = 500) -> int:
        wp = WorldPropsC(props.gravity, props.border_damping, props.cfl, props.solve_error)
        out = ctypes.c_uint64(0)
        _check(self._lib.apic_server_submit(self._h, ctypes.byref(scene), ctypes.byref(wp), steps, frame_deltatime,
                                            solver, rel_tol, max_iterations, ctypes.byref(out)),
               "apic_server_submit")
        return out.value

    def step(self) -> ServerRoundC:
        rd = ServerRoundC()
        _check(self._lib.apic_server_step(self._h, ctypes.byref(rd)), "apic_server_step")
        return rd

    def request(self, rid: int) -> RequestInfoC:
        info = RequestInfoC()
        _check(self._lib.apic_server_request(self._h, rid, ctypes.byref(info)), "apic_server_request")
        return info

    def result_positions(self, rid: int) -> np.ndarray:
        info = self.request(rid)
        out = np.zeros(info.result_floats, np.float32)
        _check(self._lib.apic_server_result_positions(self._h, rid, _fptr(out), out.size),
               "apic_server_result_positions")
        return out.reshape(-1, 2, 8)

    def stats(self) -> ServerStatsC:
        st = ServerStatsC()
        _check(self._lib.apic_server_get_stats(self._h, ctypes.byref(st)), "apic_server_get_stats")
        return st

    def close(self) -> None:
        if self._h:
            self._lib.apic_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
