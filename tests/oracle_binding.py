"""ctypes binding of the CPU oracle (oracle/nbody_oracle.c) and of the runner of
the reference's own kernel (oracle/ref_runner.cu + oracle/_ref/*.cubin).

Test infrastructure: used by tests/, the smoke check and the CPU-baseline leg of
bench.py only.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"
PORT_LIB = ROOT / "oracle" / "libcpu_port.so"
REF_DIR = ROOT / "oracle" / "_ref"
REF_CUBIN = REF_DIR / "simulator_sm103a.cubin"
REF_RUNNER = REF_DIR / "libref_runner.so"

BRANCH = 0
PREDICATED = 1

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not ORACLE_LIB.exists():
            raise RuntimeError(f"{ORACLE_LIB} missing: run `make -C oracle`")
        L = C.CDLL(str(ORACLE_LIB))
        L.oracle_step_fp32.argtypes = [C.c_int64] + [_F] * 10 + [C.c_float] * 4 + [C.c_int]
        L.oracle_run_fp32.argtypes = [C.c_int64] + [_F] * 7 + [C.c_float] * 4 + [C.c_int, C.c_int,
                                                                                _F]
        L.oracle_accel_fp32.argtypes = [C.c_int64] + [_F] * 4 + [C.c_float, C.c_float, C.c_int,
                                                                  _I64, C.c_int64] + [_F] * 3
        L.oracle_accel_fp64.argtypes = [C.c_int64] + [_F] * 4 + [C.c_double, C.c_double, _I64,
                                                                  C.c_int64] + [_D] * 3
        L.oracle_energy_fp64.argtypes = [C.c_int64] + [_F] * 7 + [C.c_double, C.c_double, _D]
        L.oracle_num_threads.restype = C.c_int
        L.oracle_set_num_threads.argtypes = [C.c_int]
        L.oracle_set_num_threads.restype = None
        L.oracle_render.argtypes = [C.c_int64] + [_F] * 7 + [C.c_int, C.c_int, _F, _F, C.c_int,
                                                              _F, C.c_int, _F]
        L.oracle_render.restype = C.c_int
        L.workload_plummer.argtypes = [C.c_uint64, C.c_uint64] + [_F] * 7
        L.workload_plummer.restype = C.c_int
        _lib = L
    return _lib


_port = None


def port() -> C.CDLL:
    """The timed CPU port (oracle/cpu_port.c, built -O3 -ffast-math -fopenmp)."""
    global _port
    if _port is None:
        if not PORT_LIB.exists():
            raise RuntimeError(f"{PORT_LIB} missing: run `make -C oracle`")
        L = C.CDLL(str(PORT_LIB))
        L.cpu_port_accel.argtypes = [C.c_int64] + [_F] * 3 + [C.c_float, C.c_float, _I64,
                                                              C.c_int64] + [_F] * 3
        L.cpu_port_accel.restype = None
        L.cpu_port_num_threads.restype = C.c_int
        L.cpu_port_set_num_threads.argtypes = [C.c_int]
        L.cpu_port_set_num_threads.restype = None
        _port = L
    return _port


def port_accel(pos, G, eps, rows=None):
    """G times the force sum of `rows` (all when None), unit masses, by the timed port."""
    x, y, z = (_f(a) for a in pos)
    r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int64)
    cnt = x.size if r is None else r.size
    out = [np.empty(cnt, dtype=np.float32) for _ in range(3)]
    port().cpu_port_accel(x.size, _p(x), _p(y), _p(z), G, eps,
                          None if r is None else r.ctypes.data_as(_I64),
                          -1 if r is None else r.size, *[_p(o) for o in out])
    return out


def port_set_num_threads(n: int) -> None:
    port().cpu_port_set_num_threads(int(n))


def port_num_threads() -> int:
    return port().cpu_port_num_threads()


def plummer(seed: int, n: int):
    """The workload's seeded Plummer sphere (oracle/workload_ic.c):
    ([x, y, z], [vx, vy, vz], mass), float32."""
    o = [np.empty(n, dtype=np.float32) for _ in range(7)]
    if lib().workload_plummer(seed, n, *[_p(a) for a in o]) != 0:
        raise MemoryError("workload_plummer")
    return o[:3], o[3:6], o[6]


def _f(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a):
    return None if a is None else a.ctypes.data_as(_F)


def num_threads() -> int:
    return lib().oracle_num_threads()


def set_num_threads(n: int) -> None:
    lib().oracle_set_num_threads(int(n))


def run_fp32(pos, vel, mass, G, dt, damping, eps, iters, method=BRANCH):
    """`iters` reference iterations; returns [x, y, z, vx, vy, vz] (new arrays)."""
    x, y, z = (_f(a).copy() for a in pos)
    vx, vy, vz = (_f(a).copy() for a in vel)
    m = None if mass is None else _f(mass)
    n = x.size
    scratch = np.empty(3 * n, dtype=np.float32)
    lib().oracle_run_fp32(n, _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(m), G, dt, damping,
                          eps, method, iters, _p(scratch))
    return [x, y, z, vx, vy, vz]


def accel_fp32(pos, mass, G, eps, rows=None, method=BRANCH):
    x, y, z = (_f(a) for a in pos)
    m = None if mass is None else _f(mass)
    r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int64)
    cnt = x.size if r is None else r.size
    out = [np.empty(cnt, dtype=np.float32) for _ in range(3)]
    lib().oracle_accel_fp32(x.size, _p(x), _p(y), _p(z), _p(m), G, eps, method,
                            None if r is None else r.ctypes.data_as(_I64),
                            -1 if r is None else r.size, *[_p(o) for o in out])
    return out


def accel_fp64(pos, mass, G, eps, rows=None):
    x, y, z = (_f(a) for a in pos)
    m = None if mass is None else _f(mass)
    r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int64)
    cnt = x.size if r is None else r.size
    out = [np.empty(cnt, dtype=np.float64) for _ in range(3)]
    lib().oracle_accel_fp64(x.size, _p(x), _p(y), _p(z), _p(m), G, eps,
                            None if r is None else r.ctypes.data_as(_I64),
                            -1 if r is None else r.size, *[o.ctypes.data_as(_D) for o in out])
    return out


def energy_fp64(pos, vel, mass, G, eps) -> dict:
    x, y, z = (_f(a) for a in pos)
    vx, vy, vz = (_f(a) for a in vel)
    m = None if mass is None else _f(mass)
    out = np.zeros(9, dtype=np.float64)
    lib().oracle_energy_fp64(x.size, _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(m), G, eps,
                             out.ctypes.data_as(_D))
    return {"kinetic": out[0], "potential": out[1], "total": out[0] + out[1],
            "momentum": list(out[2:5]), "angular_momentum": list(out[5:8]), "mass": out[8]}


def render(pos, vel, pv, width, height, offsets, weights, flare):
    """CPU restatement of the reference's render math; (height, width, 4) float32."""
    x, y, z = (_f(a) for a in pos)
    vx, vy, vz = (_f(a) for a in vel)
    pvm = _f(pv)
    off, wt, fl = _f(offsets), _f(weights), _f(flare)
    out = np.zeros((height, width, 4), np.float32)
    rc = lib().oracle_render(x.size, _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(pvm), width,
                             height, _p(off), _p(wt), off.size, _p(fl), int(round(fl.size ** 0.5)),
                             _p(out))
    if rc != 0:
        raise MemoryError("oracle_render")
    return out


# ------------------------------------------------------------------ reference kernel
def reference_available() -> bool:
    return REF_CUBIN.exists() and REF_RUNNER.exists()


def reference_run(pos, vel, G, dt, damping, eps, iters, method=BRANCH, gw_size=64):
    """Run the reference's particle_interaction (from its own source, compiled to
    a cubin) on the GPU; returns ([x, y, z, vx, vy, vz], ms)."""
    R = C.CDLL(str(REF_RUNNER))
    R.ref_run.argtypes = [C.c_char_p, C.c_int, C.c_int64] + [_F] * 6 + [
        C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, _F, C.c_char_p, C.c_int]
    R.ref_run.restype = C.c_int
    x, y, z = (_f(a).copy() for a in pos)
    vx, vy, vz = (_f(a).copy() for a in vel)
    ms = C.c_float()
    err = C.create_string_buffer(512)
    rc = R.ref_run(str(REF_CUBIN).encode(), method, x.size, _p(x), _p(y), _p(z), _p(vx), _p(vy),
                   _p(vz), iters, G, dt, damping, eps, gw_size, C.byref(ms), err, 512)
    if rc != 0:
        raise RuntimeError(f"reference kernel failed: {err.value.decode()}")
    return [x, y, z, vx, vy, vz], ms.value
