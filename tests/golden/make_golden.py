"""Generate golden vectors from the reference's own kernel.

    python tests/golden/make_golden.py [OUTDIR]      (needs a GB300)

Runs particle_interaction<BRANCH|PREDICATED> from src/simulator.cu (compiled,
unmodified, into oracle/_ref/simulator_sm103a.cubin by oracle/build_ref.sh) on
small seeded inputs and writes one .npz per case: the inputs, the parameters and
the reference kernel's outputs.  tests/test_golden_cpu.py checks the CPU oracle
against these files; tests/test_parity_gpu.py checks the library against them.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "cuda-to-sycl-nbody_gb300"))
sys.path.insert(0, str(ROOT / "tests"))

import nbody_gb300 as nb  # noqa: E402
import oracle_binding as orc  # noqa: E402


def disk(n, seed):
    (x, y, z), (vx, vy, vz), m = nb.thin_disk(seed, n, 1e-3)
    return [x, y, z], [vx, vy, vz], m


def cases():
    f32 = np.float32
    # 1. the reference's own initial state and default parameters (one stepSim)
    (x, y, z), (vx, vy, vz) = nb.reference_disk(1024)
    yield ("reference_default_n1024", [x, y, z], [vx, vy, vz],
           dict(G=2.0, dt=float(f32(0.005)), damping=float(f32(0.999998)),
                eps=float(f32(1e-7)), method=0, iters=4, gw=64))
    # 2. the perf-test argument set (scripts/perf_test_cuda.sh:17) on 5 x 256 particles
    (x, y, z), (vx, vy, vz) = nb.reference_disk(1280)
    yield ("perf_args_n1280", [x, y, z], [vx, vy, vz],
           dict(G=2.0, dt=float(f32(0.001)), damping=float(f32(0.999)), eps=float(f32(1e-3)),
                method=0, iters=5, gw=128))
    # 3. thin disk (N = 2,048), m = 1/N folded into G (10 iterations)
    pos, vel, m = disk(2048, 2024)
    yield ("thin_disk_n2048", pos, vel,
           dict(G=float(f32(1.0) * m[0]), dt=float(f32(1e-3)), damping=float(f32(0.999)),
                eps=float(f32(1e-3)), method=0, iters=10, gw=64))
    # 4. force sums: damping 0, dt 1, G 1 makes v' the kernel's force accumulator
    pos, _, _ = disk(1000, 77)
    zeros = [np.zeros(1000, np.float32)] * 3
    yield ("force_sum_n1000", pos, zeros,
           dict(G=1.0, dt=1.0, damping=0.0, eps=float(f32(1e-3)), method=0, iters=1, gw=64))
    # 5. the PREDICATED variant as shipped
    pos, vel, m = disk(512, 5)
    yield ("predicated_n512", pos, vel,
           dict(G=2.0, dt=float(f32(1e-3)), damping=float(f32(0.999)), eps=float(f32(1e-3)),
                method=1, iters=2, gw=512))
    # 6. ragged size (not a multiple of the work-group size)
    pos, vel, m = disk(333, 9)
    yield ("ragged_n333", pos, vel,
           dict(G=float(f32(1.0) * m[0]), dt=float(f32(1e-3)), damping=float(f32(0.999)),
                eps=float(f32(1e-3)), method=0, iters=3, gw=64))


def main() -> int:
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE
    out.mkdir(parents=True, exist_ok=True)
    if not orc.reference_available():
        print("reference cubin not built; run oracle/build_ref.sh on a machine with the reference")
        return 1
    cubin_sha = hashlib.sha256(orc.REF_CUBIN.read_bytes()).hexdigest()
    index = {}
    for name, pos, vel, p in cases():
        res, _ = orc.reference_run(pos, vel, p["G"], p["dt"], p["damping"], p["eps"], p["iters"],
                                   method=p["method"], gw_size=p["gw"])
        np.savez_compressed(out / f"{name}.npz", x=pos[0], y=pos[1], z=pos[2], vx=vel[0],
                            vy=vel[1], vz=vel[2], out_x=res[0], out_y=res[1], out_z=res[2],
                            out_vx=res[3], out_vy=res[4], out_vz=res[5],
                            params=json.dumps(p))
        index[name] = p
        print(name, "written")
    (out / "index.json").write_text(json.dumps({"cubin_sha256": cubin_sha, "cases": index},
                                               indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
