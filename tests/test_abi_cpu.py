"""CPU tests of the C ABI: the library loads, exports every declared symbol,
and its host logic (parameters, argv parsing, initial conditions, work-list
planning, error reporting without a GPU) behaves as specified."""
from __future__ import annotations

import math
import re
from pathlib import Path

import numpy as np
import pytest

import nbody_gb300 as nb

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "nbody_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_functions():
    names = declared_functions()
    assert len(names) >= 40
    assert "nb_sim_create" in names and "nb_sim_step" in names


def test_library_exports_every_declared_symbol():
    missing = [n for n in declared_functions() if not hasattr(nb.lib, n)]
    assert not missing, f"symbols declared in include/nbody_gb300.h but not exported: {missing}"


def test_binding_covers_every_declared_symbol():
    assert set(declared_functions()) == set(nb.SIGNATURES)


def test_abi_version_and_status_strings():
    assert nb.lib.nb_abi_version() == 1
    for code, name in [(0, "NB_OK"), (1, "NB_ERR_INVALID_ARGUMENT"), (4, "NB_ERR_NO_DEVICE"),
                       (5, "NB_ERR_DEVICE_TIMEOUT")]:
        assert nb.lib.nb_status_string(code).decode() == name


def test_simparam_defaults_match_reference():
    # SimParam::SimParam, src/sim_param.cpp:12-22
    p = nb.SimParam()
    assert p.G == 2.0
    assert p.dt == np.float32(0.005)
    assert p.numParticles == 50 * 256
    assert p.numFrames == 2 ** 64 - 1
    assert p.simIterationsPerFrame == 4
    assert p.damping == np.float32(0.999998)
    assert p.distEps == np.float32(1.0e-7)
    assert p.gwSize == 64
    assert p.calcMethod == nb.BRANCH


def test_parse_args_positional_like_reference():
    # SimParam::parseArgs, src/sim_param.cpp:40-67; the perf-test argument set
    # of scripts/perf_test_cuda.sh:17.
    p = nb.SimParam()
    p.parseArgs(["nbody", "50", "5", "0.999", "0.001", "1.0e-3", "2.0"])
    assert p.numParticles == 12800
    assert p.simIterationsPerFrame == 5
    assert p.damping == np.float32(0.999)
    assert p.dt == np.float32(0.001)
    assert p.distEps == np.float32(1e-3)
    assert p.G == 2.0
    p.parseArgs(["nbody", "4", "1", "1", "0.01", "0", "1", "7", "128", "PREDICATED"])
    assert (p.numParticles, p.numFrames, p.gwSize, p.calcMethod) == (1024, 7, 128, nb.PREDICATED)


def test_parse_args_rejects_unknown_method():
    p = nb.SimParam()
    with pytest.raises(ValueError, match="BRANCH or PREDICATED"):
        p.parseArgs(["nbody", "1", "1", "1", "1", "1", "1", "1", "64", "SIDEWAYS"])


def test_no_device_is_reported_not_fatal():
    pytest.importorskip("torch")
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(nb.NbError) as e:
        nb.device_name()
    assert e.value.status == nb.NB_ERR_NO_DEVICE
    for fn in (nb.fp32_peak_tflops, nb.measured_fp32_peak_tflops):
        with pytest.raises(nb.NbError) as e:
            fn()
        assert e.value.status == nb.NB_ERR_NO_DEVICE
    assert nb.lib.nb_measure_fp32_peak_tflops(None) == nb.NB_ERR_INVALID_ARGUMENT
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(1, 32, 1e-3)
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(nb.SimParam(numParticles=32), (x, y, z), (vx, vy, vz), m)
    assert e.value.status == nb.NB_ERR_NO_DEVICE


def test_invalid_arguments_rejected_before_device():
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(1, 32, 1e-3)
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(nb.SimParam(numParticles=32, distEps=-1.0), (x, y, z), (vx, vy, vz), m)
    assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(nb.SimParam(numParticles=32, calcMethod=7), (x, y, z), (vx, vy, vz), m)
    assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(nb.SimParam(), (x, y, z), (vx, vy, vz), m, sizes=[16, 0, 16])
    assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
    with pytest.raises(nb.NbError) as e:
        nb.Simulation(nb.SimParam(numParticles=32, accumulator=3), (x, y, z), (vx, vy, vz), m)
    assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
    assert "NB_ACC_REFERENCE_ORDER" in nb.lib.nb_last_error().decode()


def test_alloc_failure_hook_arguments():
    with pytest.raises(nb.NbError) as e:
        nb.inject_alloc_failure(-1)
    assert e.value.status == nb.NB_ERR_INVALID_ARGUMENT
    nb.inject_alloc_failure(0)                          # disarmed: a no-op


# ----------------------------------------------------------------- initial conditions
def test_thin_disk_is_deterministic_and_shaped():
    a = nb.thin_disk(5, 4096, 1e-3)
    b = nb.thin_disk(5, 4096, 1e-3)
    for u, v in zip(a[0] + a[1], b[0] + b[1]):
        assert np.array_equal(u, v)
    (x, y, z), (vx, vy, vz), m = a
    r = np.hypot(x, y)
    assert r.max() <= 1.0 + 1e-6
    assert abs(np.mean(r ** 2) - 0.5) < 0.02          # r = sqrt(u): r^2 uniform on [0, 1]
    assert abs(np.std(z) - 0.01) < 0.001               # z ~ N(0, 0.01^2)
    assert np.allclose(m, 1.0 / 4096)
    # tangential speed r * sqrt(n m r^2 / (r^2 + eps)^1.5) plus N(0, 0.01) jitter
    vt = (-y * vx + x * vy) / np.maximum(r, 1e-12)
    want = r * np.sqrt(r ** 2 / (r ** 2 + 1e-3) ** 1.5)
    assert np.std(vt - want) < 0.02
    c = nb.thin_disk(6, 4096, 1e-3)
    assert not np.array_equal(a[0][0], c[0][0])


def test_plummer_moments():
    (x, y, z), (vx, vy, vz), m = nb.plummer(3, 20000)
    assert np.isclose(m.sum(), 1.0, rtol=1e-5)
    for a in (x, y, z, vx, vy, vz):
        assert abs(float(np.mean(a))) < 1e-6             # centre of mass at rest at the origin
    r = np.sqrt(x.astype(np.float64) ** 2 + y ** 2 + z ** 2)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.305
    assert abs(np.median(r) - 1.305) < 0.05
    # virial equilibrium: 2 KE ~ -PE = 3 pi / 32 for G = M = a = 1 (untruncated)
    ke = 0.5 * np.sum(m * (vx.astype(np.float64) ** 2 + vy ** 2 + vz ** 2))
    assert abs(2 * ke - 3 * math.pi / 32) < 0.02


def test_two_disks_geometry():
    (x, y, z), (vx, vy, vz), m = nb.two_disks(2, 8192, 1e-3)
    h = 4096
    assert abs(np.mean(x[:h]) + 2.0) < 0.02 and abs(np.mean(x[h:]) - 2.0) < 0.02
    assert abs(np.mean(vx[:h]) - 0.3) < 0.05 and abs(np.mean(vx[h:]) + 0.3) < 0.05
    # the second disk is tilted by 30 degrees about the x axis: z ~ tan(30) y
    slope = np.polyfit(y[h:], z[h:], 1)[0]
    assert abs(slope - math.tan(math.radians(30))) < 0.02
    assert np.allclose(m, 1.0 / h)


def test_ensemble_sizes_log_uniform():
    s = nb.ensemble_sizes(11, 4096, 64, 8192)
    assert s.min() >= 64 and s.max() <= 8192
    logs = np.log(s.astype(np.float64))
    assert abs(np.mean(logs) - 0.5 * (math.log(64) + math.log(8192))) < 0.1
    assert 5.5e6 < s.sum() < 8.5e6                       # ~7M particles in total


def test_reference_disk_matches_reference_generator():
    # DiskGalaxySimulator::randomParticlePos / initialParticleVel
    # (simulator.cu:131-158), restated independently here with numpy's MT19937.
    n = 64
    (x, y, z), (vx, vy, vz) = nb.reference_disk(n)
    mt = np.random.RandomState(5489)                   # std::mt19937 default seed
    words = mt.randint(0, 2 ** 32, size=6 * n, dtype=np.uint64)

    def canon(k):  # std::generate_canonical<double, 53> from two 32-bit words
        return (float(words[2 * k]) + float(words[2 * k + 1]) * 2.0 ** 32) / 2.0 ** 64

    pi = float(np.float32(math.pi))
    for i in range(n):
        t = np.float32(canon(2 * i) * 2 * pi)
        s = np.float32(canon(2 * i + 1) * 100)
        assert np.isclose(x[i], np.float32(np.cos(t, dtype=np.float32) * s), rtol=2e-7, atol=1e-5)
        assert np.isclose(y[i], np.float32(np.sin(t, dtype=np.float32) * s), rtol=2e-7, atol=1e-5)
    for i in range(n):
        assert z[i] == np.float32(4.0 * canon(2 * n + i))
    speed = np.sqrt(vx.astype(np.float64) ** 2 + vy ** 2 + vz ** 2)
    rxy = np.sqrt(x.astype(np.float64) ** 2 + y ** 2)
    assert np.allclose(speed, np.sqrt(2 * rxy), rtol=1e-5)
    assert np.allclose(x * vx + y * vy, 0.0, atol=1e-2)


# ----------------------------------------------------------------- work-list planner
def _live_slots(rows, threads, r):
    # Register slots the tuned kernel runs for an i-tile with `rows` particles
    # (live_slots in csrc/nb_internal.hpp): ceil(rows / threads), capped at r, raised
    # to r when above 4.
    live = max(1, -(-rows // threads))
    return r if live >= r else (live if live <= 4 else r)


@pytest.mark.parametrize("sizes,cfg,grid", [
    ([1048576], 0, 304), ([25600], 0, 456), ([1], 0, 304), ([17], 3, 8), ([5000], 4, 7),
    ([64, 100, 8192, 3, 700], 3, 304), ([1000] * 50, 4, 152), ([100, 3000, 70, 9000], 2, 40),
    ([100, 300, 70, 2000], 1, 40), ("ensemble", 9, 152),
    ([64, 100, 8192, 3, 700], -1, 60), ([1048576], -1, 152), ([25600], -3, 152)])
def test_plan_work_covers_every_tile_once(sizes, cfg, grid):
    if sizes == "ensemble":  # 300 systems of the ensemble workload's size distribution
        sizes = [int(n) for n in nb.ensemble_sizes(20261203, 300, 64, 8192)]
    info = nb.kernel_config_info(cfg)
    threads, r = info["threads_per_block"], info["particles_per_thread"]
    bi = threads * r
    bj = info["j_tile"]
    g, segs, begin, nfix, slots = nb.plan_work(sizes, cfg, grid)
    assert 1 <= g <= grid
    assert begin[0] == 0 and begin[-1] == len(segs) and np.all(np.diff(begin) >= 0)
    covered = {}
    cost = np.zeros(g, dtype=np.int64)
    npad = [(n + 15) // 16 * 16 for n in sizes]
    # The tuned kernel's live-slot variant, and its weights, where it saves >= 1 % of
    # the slot work (live_slots_pay in csrc/worklist.hpp); the reference-order kernel
    # (cfg < 0) runs every slot.
    def live_total(n):
        full, rem = divmod(n, bi)
        return r * full + (_live_slots(rem, threads, r) if rem else 0)
    every = sum(p * r * -(-n // bi) for n, p in zip(sizes, npad))
    live = cfg >= 0 and sum(p * live_total(n) for n, p in zip(sizes, npad)) < 0.99 * every
    if len(sizes) == 300 or sizes == [100, 300, 70, 2000]:
        assert live  # these cases exercise the weighted plan
    for c in range(g):
        for sys_, it, j0, j1, fix, part in segs[begin[c]:begin[c + 1]]:
            assert j0 < j1
            for jt in range(j0, j1):
                key = (sys_, it, jt)
                assert key not in covered
                covered[key] = c
                w = _live_slots(sizes[sys_] - it * bi, threads, r) if live else 1
                cost[c] += min(bj, npad[sys_] - jt * bj) * w
    want = {(s, it, jt) for s, n in enumerate(sizes) for it in range((n + bi - 1) // bi)
            for jt in range((npad[s] + bj - 1) // bj)}
    assert set(covered) == want
    # balance: every CTA within one block of the mean charge
    assert cost.max() - cost.min() <= 2 * bj * (r if live else 1)
    # fixups: parts of a split i-tile are numbered 0.. in j order
    parts = {}
    for sys_, it, j0, j1, fix, part in segs:
        if fix >= 0:
            parts.setdefault(fix, []).append((j0, part))
    assert len(parts) == nfix
    assert sum(len(v) for v in parts.values()) == slots
    for v in parts.values():
        assert [p for _, p in sorted(v)] == list(range(len(v)))


# The fixed tables of nb_accelerations_noalloc (csrc/noalloc.cu): kernel shape 0,
# at most 262,144 particles (512 i-tiles of 512) on at most 608 persistent CTAs.
NOALLOC_CFG, NOALLOC_MAX_N, NOALLOC_MAX_GRID = 0, 262144, 608
NOALLOC_MAX_SEGMENTS = NOALLOC_MAX_SLOTS = 512 + NOALLOC_MAX_GRID - 1
NOALLOC_MAX_FIXUPS = 512


def _plan_counts(n, cfg, grid):
    import ctypes as C

    sz = np.array([n], dtype=np.uint32)
    g, nseg, nfix, slots = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    assert nb.lib.nb_plan_work(1, sz.ctypes.data_as(C.POINTER(C.c_uint32)), cfg, grid, None, 0,
                               None, C.byref(g), C.byref(nseg), C.byref(nfix),
                               C.byref(slots)) == nb.NB_OK
    return g.value, nseg.value, nfix.value, slots.value


def test_plan_size_bounds_hold_for_every_grid_of_the_noalloc_tables():
    """Replays the planner of every launch (the one nb_accelerations_noalloc uses,
    into its fixed tables) for each grid up to the entry point's cap, at the
    maximum size and at sizes whose plans are the most fragmented, and checks the
    bounds the fixed tables are sized by: segments <= i-tiles + grid - 1, slots <=
    segments, fixups <= min(i-tiles, grid - 1)."""
    info = nb.kernel_config_info(NOALLOC_CFG)
    bi = info["threads_per_block"] * info["particles_per_thread"]
    sizes = [NOALLOC_MAX_N, NOALLOC_MAX_N - 1, 214356, 131072 + 17, 65536, 12962, 5003, 513,
             512, 17, 1]
    for n in sizes:
        nit = (n + bi - 1) // bi
        for grid in range(1, NOALLOC_MAX_GRID + 1):
            g, nseg, nfix, slots = _plan_counts(n, NOALLOC_CFG, grid)
            assert g <= grid
            assert nseg <= nit + g - 1, (n, grid, nseg)
            assert slots <= nseg and nfix <= min(nit, g - 1), (n, grid, slots, nfix)
            assert nseg <= NOALLOC_MAX_SEGMENTS and slots <= NOALLOC_MAX_SLOTS
            assert nfix <= NOALLOC_MAX_FIXUPS


def test_null_handles_are_rejected_without_touching_the_device():
    import ctypes as C

    h = None
    L = nb.lib
    one = [(L.nb_sim_step, (h,)), (L.nb_sim_advance, (h, 1)),
           (L.nb_sim_advance_per_system, (h, 1)), (L.nb_sim_synchronize, (h,)),
           (L.nb_sim_inject_wait_timeout, (h,)), (L.nb_sim_inject_failure, (h, 1)),
           (L.nb_sim_generate, (h, 1, 1)),
           (L.nb_sim_get_state, (h,) + (None,) * 6), (L.nb_sim_set_state, (h,) + (None,) * 7),
           (L.nb_sim_accelerations, (h, None, None, None)),
           (L.nb_sim_set_stream, (h, None)), (L.nb_sim_export_device, (h, None, None)),
           (L.nb_sim_set_kernel_config, (h, 0)), (L.nb_sim_autotune, (h, None)),
           (L.nb_sim_graph_capture, (h, 1)), (L.nb_sim_graph_launch, (h,)),
           (L.nb_sim_diagnostics, (h, -1, None)),
           (L.nb_sim_fp64_accelerations, (h, None, 1, None, None, None)),
           (L.nb_sim_adjoint_forward, (h, 1, 1)),
           (L.nb_sim_adjoint_backward, (h, None, None, None, None)),
           (L.nb_sim_adjoint_backward_device, (h, None, None, None, None)),
           (L.nb_sim_set_shard, (h, 0, 0)), (L.nb_sim_state_block_bytes, (h, 0, 16, 1, None)),
           (L.nb_sim_copy_state_block, (h, 0, 16, 1, None)),
           (L.nb_sim_load_state_block, (h, 0, 16, 1, None)),
           (L.nb_sim_render, (h, None, None, 64, 64, None)),
           (L.nb_sim_time_iterations, (h, 1, 0, None))]
    for fn, args in one:
        assert fn(*args) == nb.NB_ERR_INVALID_ARGUMENT, fn.__name__
    out = C.c_uint64()
    assert L.nb_sim_num_particles(None, C.byref(out)) == nb.NB_ERR_INVALID_ARGUMENT
    assert L.nb_sim_destroy(None) == nb.NB_OK          # like free(NULL)
    assert L.nb_accelerations_noalloc(None, 1, 1.0, 1e-3, None, None) == \
        nb.NB_ERR_INVALID_ARGUMENT
    assert "NULL" in L.nb_last_error().decode()


@pytest.mark.parametrize("n,cfg,grid", [(1 << 20, -1, 152), (262144, -1, 152), (300000, -1, 152),
                                        (262144, -2, 456), (1 << 20, -2, 608), (200000, -2, 304),
                                        (150000, -3, 304), (25600, -4, 152), (65536, -4, 304)])
def test_ordered_hand_over_schedule_never_waits(n, cfg, grid):
    """The reference-order kernel's schedule, replayed on its own work list (shape
    -1 - cfg, unit cost per j-tile): each CTA walks its segments last to first, and the part of
    a split i-tile may start only when the previous part has finished.  With at most
    one CTA per i-tile (the kernel's grid rule) no part waits and no i-tile is split
    into more than two parts."""
    info = nb.kernel_config_info(cfg)
    bi = info["threads_per_block"] * info["particles_per_thread"]
    assert grid <= -(-n // bi)
    g, segs, begin, nfix, slots = nb.plan_work([n], cfg, grid)
    finish = {}
    for c in range(g):
        t = 0
        for q in range(begin[c + 1] - 1, begin[c] - 1, -1):
            _, _, j0, j1, fix, part = segs[q]
            if fix >= 0 and part > 0:
                assert finish[(fix, part - 1)] <= t, (c, fix, part)
            t += j1 - j0
            if fix >= 0:
                finish[(fix, part)] = t
    assert all(part <= 1 for *_, part in segs)
