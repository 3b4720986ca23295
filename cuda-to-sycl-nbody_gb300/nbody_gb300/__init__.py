"""Python binding of the GB300 n-body C ABI (include/nbody_gb300.h), via ctypes.

Mirrors the reference's simulator interface (codeplaysoftware/cuda-to-sycl-nbody):
``SimParam`` (src/sim_param.hpp:16-40) and ``DiskGalaxySimulator``
(src/simulator.cuh:129-160), plus the GB300 additions (ensembles, FP64
diagnostics, the adjoint, CUDA graphs, kernel autotuning).

Every call goes to libnbody_gb300.so; there is no CPU fallback.  Importing
this module fails if the library has not been built (``build.py``).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libnbody_gb300.so"
DRIVER_PATH = _HERE / "nbody_gb300"

NB_OK = 0
NB_ERR_INVALID_ARGUMENT = 1
NB_ERR_CUDA = 2
NB_ERR_OUT_OF_MEMORY = 3
NB_ERR_NO_DEVICE = 4
NB_ERR_DEVICE_TIMEOUT = 5
NB_ERR_STATE = 6

BRANCH = 0
PREDICATED = 1
ACC_PLAIN = 0
ACC_COMPENSATED = 1
ACC_REFERENCE_ORDER = 2
BLOCK_POSITIONS = 1
BLOCK_VELOCITIES = 2
INJECT_TILE_NEVER_COPIED = 1
INJECT_HAND_OVER_WITHHELD = 2
IC_THIN_DISK = 1
IC_PLUMMER = 2
IC_TWO_DISKS = 3


class NbError(RuntimeError):
    """A C-ABI call returned a status other than NB_OK."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{_status_name(status)}: {message}")
        self.status = status


class nb_params(C.Structure):
    _fields_ = [("G", C.c_float), ("dt", C.c_float), ("damping", C.c_float),
                ("dist_eps", C.c_float), ("num_particles", C.c_uint64),
                ("num_frames", C.c_uint64), ("iters_per_frame", C.c_int32),
                ("gw_size", C.c_int32), ("calc_method", C.c_int32), ("accumulator", C.c_int32)]


class nb_diagnostics(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("potential", C.c_double), ("total", C.c_double),
                ("momentum", C.c_double * 3), ("angular_momentum", C.c_double * 3),
                ("mass", C.c_double)]


class nb_kernel_info(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("config_index", "threads_per_block",
                                          "particles_per_thread", "j_tile", "stages", "grid",
                                          "segments", "split_tiles", "live_slots")]


class nb_segment(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("system", "i_tile", "j_tile_begin", "j_tile_end",
                                          "fixup", "part")]


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          f"`python {_HERE.parent / 'build.py'}` (needs nvcc)")
    return C.CDLL(str(LIB_PATH))


lib = _load()

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_U32 = C.POINTER(C.c_uint32)
_U64 = C.POINTER(C.c_uint64)

# name -> (restype, argtypes); every symbol declared in include/nbody_gb300.h.
SIGNATURES = {
    "nb_last_error": (C.c_char_p, []),
    "nb_status_string": (C.c_char_p, [C.c_int]),
    "nb_abi_version": (C.c_int, []),
    "nb_params_default": (None, [C.POINTER(nb_params)]),
    "nb_params_parse_args": (C.c_int, [C.POINTER(nb_params), C.c_int, C.POINTER(C.c_char_p)]),
    "nb_device_name": (C.c_int, [C.c_char_p, C.c_size_t]),
    "nb_device_fp32_peak_tflops": (C.c_int, [_D]),
    "nb_measure_fp32_peak_tflops": (C.c_int, [C.POINTER(C.c_double)]),
    "nb_sim_create": (C.c_int, [C.POINTER(nb_params)] + [_F] * 7 + [C.POINTER(_P)]),
    "nb_sim_create_disk_galaxy": (C.c_int, [C.POINTER(nb_params), C.POINTER(_P)]),
    "nb_ensemble_create": (C.c_int, [C.POINTER(nb_params), C.c_uint32, _U32] + [_F] * 7
                           + [C.POINTER(_P)]),
    "nb_sim_destroy": (C.c_int, [_P]),
    "nb_sim_step": (C.c_int, [_P]),
    "nb_sim_advance": (C.c_int, [_P, C.c_int32]),
    "nb_sim_advance_per_system": (C.c_int, [_P, C.c_int32]),
    "nb_sim_synchronize": (C.c_int, [_P]),
    "nb_sim_inject_wait_timeout": (C.c_int, [_P]),
    "nb_sim_inject_failure": (C.c_int, [_P, C.c_int32]),
    "nb_sim_generate": (C.c_int, [_P, C.c_int32, C.c_uint64]),
    "nb_camera_matrices": (C.c_int, [C.c_float, C.c_float, C.c_float, _F, C.c_int32, C.c_int32,
                                     _F, _F]),
    "nb_render_tables": (C.c_int, [_F, _F, _I32, _F]),
    "nb_sim_render": (C.c_int, [_P, _F, _F, C.c_int32, C.c_int32, _P]),
    "nb_sim_time_iterations": (C.c_int, [_P, C.c_int32, C.c_int32, _F]),
    "nb_sim_get_state": (C.c_int, [_P] + [_F] * 6),
    "nb_sim_set_state": (C.c_int, [_P] + [_F] * 7),
    "nb_sim_accelerations": (C.c_int, [_P] + [_F] * 3),
    "nb_sim_num_particles": (C.c_int, [_P, _U64]),
    "nb_sim_num_systems": (C.c_int, [_P, _U32]),
    "nb_sim_last_step_ms": (C.c_int, [_P, _F]),
    "nb_sim_gw_size": (C.c_int, [_P, _I32]),
    "nb_sim_calc_method": (C.c_int, [_P, _I32]),
    "nb_sim_set_stream": (C.c_int, [_P, _P]),
    "nb_sim_export_device": (C.c_int, [_P, _P, _P]),
    "nb_num_kernel_configs": (C.c_int, []),
    "nb_kernel_config_info": (C.c_int, [C.c_int32, C.POINTER(nb_kernel_info)]),
    "nb_sim_set_kernel_config": (C.c_int, [_P, C.c_int32]),
    "nb_sim_kernel_info": (C.c_int, [_P, C.POINTER(nb_kernel_info)]),
    "nb_sim_autotune": (C.c_int, [_P, _I32]),
    "nb_plan_work": (C.c_int, [C.c_uint32, _U32, C.c_int32, C.c_int32, C.POINTER(nb_segment),
                               C.c_int32, _I32, _I32, _I32, _I32, _I32]),
    "nb_inject_alloc_failure": (C.c_int, [C.c_int32]),
    "nb_sim_graph_capture": (C.c_int, [_P, C.c_int32]),
    "nb_sim_graph_launch": (C.c_int, [_P]),
    "nb_sim_diagnostics": (C.c_int, [_P, C.c_int32, C.POINTER(nb_diagnostics)]),
    "nb_sim_fp64_accelerations": (C.c_int, [_P, _U64, C.c_uint64, _D, _D, _D]),
    "nb_sim_adjoint_forward": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "nb_sim_adjoint_backward": (C.c_int, [_P] + [_F] * 4),
    "nb_sim_adjoint_backward_device": (C.c_int, [_P] * 5),
    "nb_accelerations_noalloc": (C.c_int, [_P, C.c_uint64, C.c_float, C.c_float, _P, _P]),
    "nb_sim_set_shard": (C.c_int, [_P, C.c_uint64, C.c_uint64]),
    "nb_sim_state_block_bytes": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_int32, _U64]),
    "nb_sim_copy_state_block": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_int32, _P]),
    "nb_sim_load_state_block": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_int32, _P]),
    "nb_ic_thin_disk": (C.c_int, [C.c_uint64, C.c_uint64, C.c_float] + [_F] * 7),
    "nb_ic_plummer": (C.c_int, [C.c_uint64, C.c_uint64] + [_F] * 7),
    "nb_ic_two_disks": (C.c_int, [C.c_uint64, C.c_uint64, C.c_float] + [_F] * 7),
    "nb_ic_ensemble_sizes": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, _U32]),
    "nb_ic_reference_disk": (C.c_int, [C.c_uint64] + [_F] * 6),
}

for _name, (_res, _args) in SIGNATURES.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


def _status_name(status: int) -> str:
    return lib.nb_status_string(status).decode()


def _check(status: int) -> None:
    if status != NB_OK:
        raise NbError(status, lib.nb_last_error().decode())


def _f32(a, n: int | None = None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _fp(a) -> C.POINTER(C.c_float):
    return None if a is None else a.ctypes.data_as(_F)


# ---------------------------------------------------------------------------- params
class SimParam:
    """Mirror of the reference's SimParam (src/sim_param.hpp:16-40)."""

    FIELDS = ("G", "dt", "numParticles", "numFrames", "simIterationsPerFrame", "damping",
              "distEps", "gwSize", "calcMethod")

    def __init__(self, **kw):
        p = nb_params()
        lib.nb_params_default(C.byref(p))
        self._from_c(p)
        self.accumulator = ACC_COMPENSATED  # the library default (nb_params_default)
        for k, v in kw.items():
            if k not in self.FIELDS and k != "accumulator":
                raise TypeError(f"unknown SimParam field {k}")
            setattr(self, k, v)

    def _from_c(self, p: nb_params) -> None:
        self.G, self.dt, self.damping, self.distEps = p.G, p.dt, p.damping, p.dist_eps
        self.numParticles, self.numFrames = p.num_particles, p.num_frames
        self.simIterationsPerFrame, self.gwSize = p.iters_per_frame, p.gw_size
        self.calcMethod = p.calc_method

    def to_c(self) -> nb_params:
        p = nb_params()
        p.G, p.dt, p.damping, p.dist_eps = self.G, self.dt, self.damping, self.distEps
        p.num_particles, p.num_frames = int(self.numParticles), int(self.numFrames)
        p.iters_per_frame, p.gw_size = int(self.simIterationsPerFrame), int(self.gwSize)
        p.calc_method, p.accumulator = int(self.calcMethod), int(self.accumulator)
        return p

    def parseArgs(self, argv: list[str]) -> None:
        """SimParam::parseArgs (src/sim_param.cpp:40-67); argv[0] is the program name."""
        p = self.to_c()
        arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        st = lib.nb_params_parse_args(C.byref(p), len(argv), arr)
        if st == NB_ERR_INVALID_ARGUMENT:
            raise ValueError(lib.nb_last_error().decode())
        _check(st)
        self._from_c(p)


# ---------------------------------------------------------------------------- device
def device_name() -> str:
    buf = C.create_string_buffer(256)
    _check(lib.nb_device_name(buf, 256))
    return buf.value.decode()


def fp32_peak_tflops() -> float:
    v = C.c_double()
    _check(lib.nb_device_fp32_peak_tflops(C.byref(v)))
    return v.value


def inject_alloc_failure(nth: int) -> None:
    """Test hook: the nth device allocation of the library from now on fails with
    NB_ERR_OUT_OF_MEMORY (0 disarms)."""
    _check(lib.nb_inject_alloc_failure(nth))


def measured_fp32_peak_tflops() -> float:
    """FP32 TFLOP/s of an FFMA2 loop kernel on the current device (measured)."""
    v = C.c_double()
    _check(lib.nb_measure_fp32_peak_tflops(C.byref(v)))
    return v.value


def num_kernel_configs() -> int:
    return lib.nb_num_kernel_configs()


def kernel_config_info(index: int) -> dict:
    k = nb_kernel_info()
    _check(lib.nb_kernel_config_info(index, C.byref(k)))
    return {f: getattr(k, f) for f, _ in nb_kernel_info._fields_}


def plan_work(sizes, config_index: int, max_grid: int):
    """Work list of the persistent kernel: (grid, segments (n x 6 int32), seg_begin, fixups, slots)."""
    sz = np.ascontiguousarray(sizes, dtype=np.uint32)
    grid, nseg, nfix, slots = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    _check(lib.nb_plan_work(len(sz), sz.ctypes.data_as(_U32), config_index, max_grid, None, 0,
                            None, C.byref(grid), C.byref(nseg), C.byref(nfix), C.byref(slots)))
    segs = (nb_segment * max(1, nseg.value))()
    begin = np.zeros(grid.value + 1, dtype=np.int32)
    _check(lib.nb_plan_work(len(sz), sz.ctypes.data_as(_U32), config_index, max_grid, segs,
                            nseg.value, begin.ctypes.data_as(_I32), None, None, None, None))
    arr = np.ctypeslib.as_array(C.cast(segs, _I32), shape=(max(1, nseg.value) * 6,))
    arr = arr.reshape(-1, 6)[: nseg.value].copy()
    return grid.value, arr, begin, nfix.value, slots.value


def accelerations_noalloc(pos_xyzm_ptr: int, n: int, G: float, dist_eps: float,
                          accel_xyzw_ptr: int, stream_ptr: int | None = None) -> None:
    """nb_accelerations_noalloc on caller device buffers (float4 per particle)."""
    _check(lib.nb_accelerations_noalloc(C.c_void_p(pos_xyzm_ptr), n, G, dist_eps,
                                        C.c_void_p(accel_xyzw_ptr),
                                        C.c_void_p(stream_ptr) if stream_ptr else None))


def camera_matrices(azimuth: float, elevation: float, distance: float, width: int, height: int,
                    look_at=(0.0, 0.0, 0.0)):
    """(view, proj) as 4x4 column-major float32 arrays (flattened, OpenGL order)."""
    view = np.empty(16, np.float32)
    proj = np.empty(16, np.float32)
    at = np.asarray(look_at, np.float32)
    _check(lib.nb_camera_matrices(azimuth, elevation, distance, at.ctypes.data_as(_F), width,
                                  height, view.ctypes.data_as(_F), proj.ctypes.data_as(_F)))
    return view, proj


def render_tables():
    """(gauss offsets, gauss weights, flare 16x16) of the renderer."""
    off = np.zeros(32, np.float32)
    w = np.zeros(32, np.float32)
    taps = C.c_int32()
    flare = np.zeros(256, np.float32)
    _check(lib.nb_render_tables(off.ctypes.data_as(_F), w.ctypes.data_as(_F), C.byref(taps),
                                flare.ctypes.data_as(_F)))
    return off[:taps.value], w[:taps.value], flare.reshape(16, 16)


# ---------------------------------------------------------------------------- initial conditions
def _ic_out(n: int):
    return [np.empty(n, dtype=np.float32) for _ in range(7)]


def thin_disk(seed: int, n: int, eps: float):
    o = _ic_out(n)
    _check(lib.nb_ic_thin_disk(seed, n, eps, *[_fp(a) for a in o]))
    return o[:3], o[3:6], o[6]


def plummer(seed: int, n: int):
    o = _ic_out(n)
    _check(lib.nb_ic_plummer(seed, n, *[_fp(a) for a in o]))
    return o[:3], o[3:6], o[6]


def two_disks(seed: int, n: int, eps: float):
    o = _ic_out(n)
    _check(lib.nb_ic_two_disks(seed, n, eps, *[_fp(a) for a in o]))
    return o[:3], o[3:6], o[6]


def ensemble_sizes(seed: int, count: int, lo: int, hi: int) -> np.ndarray:
    s = np.empty(count, dtype=np.uint32)
    _check(lib.nb_ic_ensemble_sizes(seed, count, lo, hi, s.ctypes.data_as(_U32)))
    return s


def reference_disk(n: int):
    o = _ic_out(n)
    _check(lib.nb_ic_reference_disk(n, *[_fp(a) for a in o[:6]]))
    return o[:3], o[3:6]


# ---------------------------------------------------------------------------- simulation
class Simulation:
    """An nb_sim handle: one system, or an ensemble of independent systems."""

    def __init__(self, params: SimParam, pos, vel, mass=None, sizes=None):
        self.params = params
        n = int(sum(int(s) for s in sizes)) if sizes is not None else int(params.numParticles)
        params.numParticles = n
        self.n = n
        x, y, z = (_f32(a, n) for a in pos)
        vx, vy, vz = (_f32(a, n) for a in vel)
        m = None if mass is None else _f32(mass, n)
        h = C.c_void_p()
        p = params.to_c()
        if sizes is None:
            _check(lib.nb_sim_create(C.byref(p), _fp(x), _fp(y), _fp(z), _fp(vx), _fp(vy),
                                     _fp(vz), _fp(m), C.byref(h)))
            self.sizes = np.array([n], dtype=np.uint32)
        else:
            self.sizes = np.ascontiguousarray(sizes, dtype=np.uint32)
            _check(lib.nb_ensemble_create(C.byref(p), len(self.sizes),
                                          self.sizes.ctypes.data_as(_U32), _fp(x), _fp(y), _fp(z),
                                          _fp(vx), _fp(vy), _fp(vz), _fp(m), C.byref(h)))
        self._h = h

    @classmethod
    def reference_disk(cls, params: SimParam) -> "Simulation":
        self = cls.__new__(cls)
        self.params = params
        self.n = int(params.numParticles)
        self.sizes = np.array([self.n], dtype=np.uint32)
        h = C.c_void_p()
        p = params.to_c()
        _check(lib.nb_sim_create_disk_galaxy(C.byref(p), C.byref(h)))
        self._h = h
        return self

    # lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.nb_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # stepping
    def step(self) -> None:
        _check(lib.nb_sim_step(self._h))

    def advance(self, iterations: int) -> None:
        _check(lib.nb_sim_advance(self._h, iterations))

    def advance_per_system(self, iterations: int) -> None:
        _check(lib.nb_sim_advance_per_system(self._h, iterations))

    def synchronize(self) -> None:
        _check(lib.nb_sim_synchronize(self._h))

    def inject_wait_timeout(self) -> None:
        """Failure-detection test hook: the next launch's bounded waits run out."""
        _check(lib.nb_sim_inject_wait_timeout(self._h))

    def inject_failure(self, kind: int) -> None:
        """Failure-detection test hook (INJECT_*) for the next force launch."""
        _check(lib.nb_sim_inject_failure(self._h, kind))

    def time_iterations(self, iterations: int, per_system: int = 0) -> float:
        """Device milliseconds of `iterations` iterations (CUDA events).  per_system:
        0 one launch over every system; 1 (or True) one launch per system with the
        shape each would get alone; 2 one launch per system with this simulation's
        shape."""
        ms = C.c_float()
        _check(lib.nb_sim_time_iterations(self._h, iterations, int(per_system), C.byref(ms)))
        return ms.value

    def last_step_ms(self) -> float:
        ms = C.c_float()
        _check(lib.nb_sim_last_step_ms(self._h, C.byref(ms)))
        return ms.value

    # state
    def get_state(self, out=None):
        o = out if out is not None else [np.empty(self.n, dtype=np.float32) for _ in range(6)]
        _check(lib.nb_sim_get_state(self._h, *[_fp(a) for a in o]))
        return o

    def set_state(self, pos=None, vel=None, mass=None) -> None:
        arrs = [None] * 6
        if pos is not None:
            arrs[0:3] = [_f32(a, self.n) for a in pos]
        if vel is not None:
            arrs[3:6] = [_f32(a, self.n) for a in vel]
        m = None if mass is None else _f32(mass, self.n)
        _check(lib.nb_sim_set_state(self._h, *[_fp(a) for a in arrs], _fp(m)))

    def generate(self, kind: int, seed: int) -> None:
        """Regenerate every system's state on the GPU (system k uses seed + k)."""
        _check(lib.nb_sim_generate(self._h, kind, seed))

    def accelerations(self):
        o = [np.empty(self.n, dtype=np.float32) for _ in range(3)]
        _check(lib.nb_sim_accelerations(self._h, *[_fp(a) for a in o]))
        return o

    def render(self, view, proj, width: int, height: int, rgba_ptr: int) -> None:
        """Render into a width x height float4 device buffer (row 0 at the bottom)."""
        v = np.ascontiguousarray(view, np.float32)
        p = np.ascontiguousarray(proj, np.float32)
        _check(lib.nb_sim_render(self._h, v.ctypes.data_as(_F), p.ctypes.data_as(_F), width,
                                 height, C.c_void_p(rgba_ptr)))

    def export_device(self, pos_ptr: int, vel_ptr: int | None = None) -> None:
        _check(lib.nb_sim_export_device(self._h, C.c_void_p(pos_ptr),
                                        C.c_void_p(vel_ptr) if vel_ptr else None))

    # shards of one system (nb_sim_set_shard); see nbody_gb300.shard
    def set_shard(self, first: int, count: int) -> None:
        _check(lib.nb_sim_set_shard(self._h, first, count))

    def state_block_bytes(self, first: int, count: int, what: int = BLOCK_POSITIONS) -> int:
        v = C.c_uint64()
        _check(lib.nb_sim_state_block_bytes(self._h, first, count, what, C.byref(v)))
        return v.value

    def copy_state_block(self, first: int, count: int, what: int, dst_ptr: int) -> None:
        _check(lib.nb_sim_copy_state_block(self._h, first, count, what, C.c_void_p(dst_ptr)))

    def load_state_block(self, first: int, count: int, what: int, src_ptr: int) -> None:
        _check(lib.nb_sim_load_state_block(self._h, first, count, what, C.c_void_p(src_ptr)))

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(lib.nb_sim_set_stream(self._h, C.c_void_p(stream_ptr) if stream_ptr else None))

    # queries
    def num_particles(self) -> int:
        v = C.c_uint64()
        _check(lib.nb_sim_num_particles(self._h, C.byref(v)))
        return v.value

    def num_systems(self) -> int:
        v = C.c_uint32()
        _check(lib.nb_sim_num_systems(self._h, C.byref(v)))
        return v.value

    def gw_size(self) -> int:
        v = C.c_int32()
        _check(lib.nb_sim_gw_size(self._h, C.byref(v)))
        return v.value

    def calc_method(self) -> int:
        v = C.c_int32()
        _check(lib.nb_sim_calc_method(self._h, C.byref(v)))
        return v.value

    # kernel selection
    def set_kernel_config(self, index: int) -> None:
        _check(lib.nb_sim_set_kernel_config(self._h, index))

    def kernel_info(self) -> dict:
        k = nb_kernel_info()
        _check(lib.nb_sim_kernel_info(self._h, C.byref(k)))
        return {f: getattr(k, f) for f, _ in nb_kernel_info._fields_}

    def autotune(self) -> int:
        """Time the kernel shapes on this simulation's data and keep the fastest.
        Returns the tuned kernel's config index, or -1 - shape for the
        reference-order kernel (NB_ACC_REFERENCE_ORDER)."""
        v = C.c_int32()
        _check(lib.nb_sim_autotune(self._h, C.byref(v)))
        return v.value

    # graphs
    def graph_capture(self, iterations: int) -> None:
        _check(lib.nb_sim_graph_capture(self._h, iterations))

    def graph_launch(self) -> None:
        _check(lib.nb_sim_graph_launch(self._h))

    # diagnostics
    def diagnostics(self, system: int = -1) -> dict:
        d = nb_diagnostics()
        _check(lib.nb_sim_diagnostics(self._h, system, C.byref(d)))
        return {"kinetic": d.kinetic, "potential": d.potential, "total": d.total,
                "momentum": list(d.momentum), "angular_momentum": list(d.angular_momentum),
                "mass": d.mass}

    def fp64_accelerations(self, rows):
        r = np.ascontiguousarray(rows, dtype=np.uint64)
        o = [np.empty(len(r), dtype=np.float64) for _ in range(3)]
        _check(lib.nb_sim_fp64_accelerations(self._h, r.ctypes.data_as(_U64), len(r),
                                             *[a.ctypes.data_as(_D) for a in o]))
        return o

    # adjoint
    def adjoint_forward(self, T: int, checkpoint_every: int) -> None:
        _check(lib.nb_sim_adjoint_forward(self._h, T, checkpoint_every))

    def adjoint_backward(self, gx_T, gv_T=None):
        gx = _f32(gx_T, 3 * self.n)
        gv = None if gv_T is None else _f32(gv_T, 3 * self.n)
        ox = np.empty(3 * self.n, dtype=np.float32)
        ov = np.empty(3 * self.n, dtype=np.float32)
        _check(lib.nb_sim_adjoint_backward(self._h, _fp(gx), _fp(gv), _fp(ox), _fp(ov)))
        return ox.reshape(self.n, 3), ov.reshape(self.n, 3)

    def adjoint_backward_device(self, gx_T_ptr: int, gv_T_ptr: int | None, gx_0_ptr: int,
                                gv_0_ptr: int) -> None:
        """nb_sim_adjoint_backward on device arrays (n x 3 float32 each), enqueued on
        the simulation's stream."""
        _check(lib.nb_sim_adjoint_backward_device(
            self._h, C.c_void_p(gx_T_ptr), C.c_void_p(gv_T_ptr) if gv_T_ptr else None,
            C.c_void_p(gx_0_ptr), C.c_void_p(gv_0_ptr)))


class DiskGalaxySimulator:
    """simulation::DiskGalaxySimulator (src/simulator.cuh:129-160) over the C ABI."""

    def __init__(self, params: SimParam, pos=None, vel=None, mass=None):
        self.params = params
        if pos is None:
            self._sim = Simulation.reference_disk(params)
        else:
            self._sim = Simulation(params, pos, vel, mass)
        self._pos = [np.empty(self._sim.n, dtype=np.float32) for _ in range(3)]
        self._vel = [np.empty(self._sim.n, dtype=np.float32) for _ in range(3)]
        self._recv()

    def _recv(self) -> None:
        self._sim.get_state(self._pos + self._vel)

    @property
    def simulation(self) -> Simulation:
        return self._sim

    def stepSim(self) -> None:
        self._sim.step()
        self._recv()  # recvFromDevice every step, src/simulator.cu:74

    def getNumParticles(self) -> int:
        return self._sim.num_particles()

    def getParticlePos(self):
        return self._pos

    def getParticleVel(self):
        return self._vel

    def getLastStepTime(self) -> float:
        return self._sim.last_step_ms()

    def getDeviceName(self) -> str:
        try:
            return device_name()
        except NbError:
            return "Unknown Device"

    def getGwSize(self) -> int:
        return self._sim.gw_size()

    def getCM(self) -> int:
        return self._sim.calc_method()
