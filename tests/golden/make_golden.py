"""Generate the golden fixtures in tests/golden/ by running the REFERENCE's own
CPU kernels and its parameter derivation (oracle/_ref/libref_cavity.so, built
from the reference checkout by ``make -C oracle ref``).

Run here, where the reference checkout exists:

    python tests/golden/make_golden.py [--ref-src /path/to/cavityflow_cuda/src]

Outputs (committed):
  * ``params.json``  -- tau, 1/tau, U*, g* per configuration XML in configs/,
    as src/CLbmSolver.cpp:28-327 derives them (float and double).
  * ``<case>.npz``   -- raw population and flag arrays after N steps for small
    cavities (reference layout, see oracle/oracle.py), plus the inputs.
  * ``digests.json`` -- for the larger runs whose arrays are too big to
    commit: sha256 of the raw population bytes, FP64 totals and centre-line
    velocity profiles.

The reference was built for x86-64, where g++ emits no fused multiply-add,
so these are the reference kernels' exact bits.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402

# (name, nx, ny, nz, dtype, nu, U, steps, gravity, lid)
SMALL_CASES = [
    ("cube8_f64", 8, 8, 8, np.float64, 0.032, 0.05, [1, 2, 7, 40], (0.0, 0.0, 0.0), True),
    ("box10x7x5_f64", 10, 7, 5, np.float64, 0.0192, 0.1, [9, 30], (0.0, 0.0, 0.0), True),
    ("cube8_f32", 8, 8, 8, np.float32, 0.032, 0.05, [1, 2, 7, 40], (0.0, 0.0, 0.0), True),
    ("box13x6x9_f32", 13, 6, 9, np.float32, 0.0512, 0.1, [11, 50], (0.0, 0.0, 0.0), True),
    ("gravity12x9x6_f32", 12, 9, 6, np.float32, 0.032, 0.05, [25], (1e-4, -2e-4, 3e-5), True),
    ("gravity9x9x9_f64", 9, 9, 9, np.float64, 0.05, 0.08, [14], (2e-4, -1e-4, 0.0), True),
    ("walls10_f64", 10, 10, 10, np.float64, 0.032, 0.05, [60], (0.0, 0.0, 0.0), False),
]

# Larger runs kept as digests: (name, nx, ny, nz, dtype, nu, U, steps)
DIGEST_CASES = [
    ("cavity64_f64_1000", 64, 64, 64, np.float64, 0.032, 0.05, 1000),
    ("cavity24_f32_1000", 24, 24, 24, np.float32, 0.0192, 0.05, 1000),
    ("box40x24x32_f32_300", 40, 24, 32, np.float32, 0.0512, 0.1, 300),
]

CONFIG_TEMPLATE = """<?xml version="1.0" encoding="ISO-8859-1"?>
<lbm-configuration>
  <physics>
    <velocity><x>{ux}</x><y>0</y><z>0</z></velocity>
    <acceleration><x>{gx}</x><y>{gy}</y><z>{gz}</z></acceleration>
    <viscosity>{nu}</viscosity>
    <max-velocity>{umax}</max-velocity>
    <max-acceleration>0.1</max-acceleration>
  </physics>
  <grid>
    <domain-size><x>{nx}</x><y>{ny}</y><z>{nz}</z></domain-size>
    <domian-length><x>{lx}</x><y>{ly}</y><z>{lz}</z></domian-length>
    <subdomain-num><x>1</x><y>1</y><z>1</z></subdomain-num>
    <cpu-subdomain-ratio>0.0</cpu-subdomain-ratio>
  </grid>
  <simulation>
    <loops>{loops}</loops>
    <timestep>{dt}</timestep>
    <benchmark><do>0</do><output-dir>benchmark</output-dir></benchmark>
    <logging><do>0</do><output-dir>log</output-dir></logging>
    <validation><do>0</do><output-dir>validation</output-dir></validation>
    <visualization><do>0</do><rate>100</rate><output-dir>visualization</output-dir></visualization>
  </simulation>
  <cpu>
    <block-configuration>
      <alpha-block-configuration><x>32</x><y>32</y><z>32</z></alpha-block-configuration>
      <beta-block-configuration><x>32</x><y>32</y><z>32</z></beta-block-configuration>
    </block-configuration>
  </cpu>
  <gpu>
    <grid-configuration>
      <init-grid-configuration><x>32</x><y>16</y><z>1</z></init-grid-configuration>
      <alpha-grid-configuration><x>32</x><y>8</y><z>1</z></alpha-grid-configuration>
      <beta-grid-configuration><x>32</x><y>8</y><z>1</z></beta-grid-configuration>
    </grid-configuration>
  </gpu>
</lbm-configuration>
"""

# Configurations whose derived lattice parameters are pinned.  The first four
# are the lid-driven cavity runs the benchmarks use (dx = dt = 1, so the
# lattice values equal the physical ones); the rest exercise the time-step
# rescaling branches of src/CLbmSolver.cpp:121-279.
CONFIGS = {
    "cavity64_re100": dict(nx=64, ny=64, nz=64, lx=64, ly=64, lz=64, ux=0.05, nu=0.032, dt=1, umax=0.1,
                           gx=0, gy=0, gz=0, loops=1000),
    "cavity384_re1000": dict(nx=384, ny=384, nz=384, lx=384, ly=384, lz=384, ux=0.05, nu=0.0192, dt=1,
                             umax=0.1, gx=0, gy=0, gz=0, loops=2000),
    "cavity512_re1000": dict(nx=512, ny=512, nz=512, lx=512, ly=512, lz=512, ux=0.1, nu=0.0512, dt=1,
                             umax=0.1, gx=0, gy=0, gz=0, loops=5000),
    "unit_box_auto_nu": dict(nx=32, ny=32, nz=32, lx=1.0, ly=1.0, lz=1.0, ux=1.0, nu=-1, dt=0.01, umax=0.1,
                             gx=0, gy=-9.81, gz=0, loops=10),
    "velocity_limited": dict(nx=48, ny=48, nz=48, lx=1.0, ly=1.0, lz=1.0, ux=2.0, nu=0.01, dt=0.05,
                             umax=0.08, gx=0, gy=0, gz=0, loops=10),
    "accel_limited": dict(nx=32, ny=32, nz=32, lx=1.0, ly=1.0, lz=1.0, ux=0.5, nu=0.02, dt=0.02,
                          umax=0.1, gx=0, gy=-9.81, gz=0, loops=10),
    "infeasible": dict(nx=48, ny=48, nz=48, lx=1.0, ly=1.0, lz=1.0, ux=2.0, nu=0.001, dt=0.05,
                       umax=0.08, gx=0, gy=0, gz=0, loops=10),
    "tau_limited": dict(nx=40, ny=40, nz=40, lx=40, ly=40, lz=40, ux=0.01, nu=0.5, dt=1, umax=0.1,
                        gx=0, gy=0, gz=0, loops=10),
}


# A configuration that sets every field of the reader to a non-default value,
# with comments and loose whitespace, for the reader's own parity test.
READER_VARIETY = """<?xml version="1.0" encoding="ISO-8859-1"?>
<!-- every field non-default -->
<lbm-configuration>
  <physics>
    <velocity>
      <x> 0.075 </x><y>0.001</y><z>-0.002</z>
    </velocity>
    <acceleration><x>0.0001</x><y>-0.0002</y><z>0.0003</z></acceleration>
    <viscosity>0.0425</viscosity>
    <max-velocity>0.09</max-velocity>
    <max-acceleration>0.05</max-acceleration>
  </physics>
  <grid>
    <domain-size><x>40</x><y>24</y><z>32</z></domain-size>
    <!-- the reference's own spelling of this tag -->
    <domian-length><x>40</x><y>24</y><z>32</z></domian-length>
    <subdomain-num><x>2</x><y>1</y><z>1</z></subdomain-num>
    <cpu-subdomain-ratio>0.25</cpu-subdomain-ratio>
  </grid>
  <simulation>
    <loops>123</loops>
    <timestep>1.0</timestep>
    <benchmark><do>1</do><output-dir>out/bench</output-dir></benchmark>
    <logging><do>1</do><output-dir>out/log</output-dir></logging>
    <validation><do>1</do><output-dir>out/valid</output-dir></validation>
    <visualization><do>1</do><rate>7</rate><output-dir>out/vis</output-dir></visualization>
  </simulation>
  <cpu>
    <block-configuration>
      <alpha-block-configuration><x>16</x><y>8</y><z>4</z></alpha-block-configuration>
      <beta-block-configuration><x>8</x><y>4</y><z>2</z></beta-block-configuration>
    </block-configuration>
  </cpu>
  <gpu>
    <grid-configuration>
      <init-grid-configuration><x>64</x><y>4</y><z>2</z></init-grid-configuration>
      <alpha-grid-configuration><x>128</x><y>2</y><z>1</z></alpha-grid-configuration>
      <beta-grid-configuration><x>256</x><y>1</y><z>1</z></beta-grid-configuration>
    </grid-configuration>
  </gpu>
</lbm-configuration>
"""


def make_config_fixtures() -> None:
    """configs.json: every field the reference's reader returns for each
    configs/*.xml, in double and in float; each read runs in its own process
    because the reference's checks assert."""
    cfg_dir = os.path.join(HERE, "configs")
    with open(os.path.join(cfg_dir, "reader_variety.xml"), "w") as fh:
        fh.write(READER_VARIETY)
    out = {}
    for f in sorted(os.listdir(cfg_dir)):
        if not f.endswith(".xml"):
            continue
        out[f[:-4]] = {}
        for tag in ("f64", "f32"):
            r = subprocess.run([sys.executable, __file__, "--config-one", os.path.join(cfg_dir, f), tag],
                               capture_output=True, text=True)
            out[f[:-4]][tag] = ({"error": True} if r.returncode != 0
                                else json.loads(r.stdout.strip().splitlines()[-1]))
    with open(os.path.join(HERE, "configs.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


def post_collision(dd: np.ndarray, last_was_alpha: bool) -> np.ndarray:
    """Interior post-collision populations f_k (19, nz, ny, nx): after alpha
    they sit swapped in the cell's own slots, after beta in slot k of x + c_k."""
    cx = [1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0]
    cy = [0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0]
    cz = [0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0]
    _, Z, Y, X = dd.shape
    out = np.empty((19, Z - 2, Y - 2, X - 2), dtype=np.float64)
    for k in range(19):
        if last_was_alpha:
            src = k ^ 1 if k < 18 else 18
            out[k] = dd[src, 1:-1, 1:-1, 1:-1]
        else:
            out[k] = dd[k, 1 + cz[k]:Z - 1 + cz[k], 1 + cy[k]:Y - 1 + cy[k], 1 + cx[k]:X - 1 + cx[k]]
    return out


def profiles(dd: np.ndarray, last_was_alpha: bool):
    """Centre-line velocities of the cavity (u = j, incompressible form):
    u_x(y) on the vertical line x = z = centre, u_y(x) on the horizontal line
    y = z = centre.  Plain numpy sums in float64 (order differs from the
    kernels', so these are compared with a tolerance)."""
    f = post_collision(dd, last_was_alpha)
    jx = f[0] - f[1] + f[4] - f[5] + f[6] - f[7] + f[8] - f[9] + f[10] - f[11]
    jy = f[2] - f[3] + f[4] - f[5] - f[6] + f[7] + f[12] - f[13] + f[14] - f[15]
    nz, ny, nx = jx.shape
    return jx[nz // 2, :, nx // 2].copy(), jy[nz // 2, ny // 2, :].copy()


def sha256(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=orc.reference_src(),
                    help="the reference checkout's src/ (default: LBM_REFERENCE_DIR/src)")
    ap.add_argument("--skip-digests", action="store_true")
    ap.add_argument("--params-one", nargs=2, metavar=("XML", "DTYPE"))
    ap.add_argument("--config-one", nargs=2, metavar=("XML", "DTYPE"))
    ap.add_argument("--configs-only", action="store_true", help="regenerate configs.json only")
    args = ap.parse_args()
    if args.config_one:
        xml, tag = args.config_one
        print(json.dumps(orc.Reference().config(xml, np.float64 if tag == "f64" else np.float32)))
        return
    if args.configs_only:
        orc.build(args.ref_src)
        make_config_fixtures()
        return
    if args.params_one:
        xml, tag = args.params_one
        v = orc.Reference().params(xml, np.float64 if tag == "f64" else np.float32)
        print(json.dumps(v.tolist()))
        return
    orc.build(args.ref_src)
    ref = orc.Reference()

    # 1. parameter derivation
    cfg_dir = os.path.join(HERE, "configs")
    os.makedirs(cfg_dir, exist_ok=True)
    params = {}
    for name, c in CONFIGS.items():
        path = os.path.join(cfg_dir, f"{name}.xml")
        with open(path, "w") as fh:
            fh.write(CONFIG_TEMPLATE.format(**c))
        params[name] = {}
        for tag in ("f64", "f32"):
            # the reference exit()s on an infeasible configuration, so each
            # probe runs in its own process
            r = subprocess.run([sys.executable, __file__, "--params-one", path, tag],
                               capture_output=True, text=True)
            if r.returncode != 0:
                params[name][tag] = {"error": True}
            else:
                v = json.loads(r.stdout.strip().splitlines()[-1])
                params[name][tag] = dict(zip(
                    ["timestep", "tau", "tau_inv", "ux", "uy", "uz", "gx", "gy", "gz", "nu"], v))
    with open(os.path.join(HERE, "params.json"), "w") as fh:
        json.dump(params, fh, indent=1, sort_keys=True)
    make_config_fixtures()

    # 2. small cases: full arrays
    for name, nx, ny, nz, dtype, nu, U, steps_list, g, lid in SMALL_CASES:
        tau, itau = orc.tau_of(nu, dtype)
        T = np.dtype(dtype).type
        out = dict(nx=nx, ny=ny, nz=nz, inv_tau=np.array(itau, dtype=dtype), lid_u=np.array(T(U), dtype=dtype),
                   gravity=np.array(g, dtype=dtype), lid=np.array(lid), steps=np.array(steps_list))
        dd, flags = ref.init(nx, ny, nz, dtype)
        out["init_dd"] = dd.copy()
        if lid:
            flags[1:-1, ny, 1:-1] = orc.VELOCITY_INJECTION
        out["flags"] = flags.copy()
        done = 0
        for n in steps_list:
            while done < n:
                ref.step(dd, flags, done, itau, T(U), tuple(T(x) for x in g))
                done += 1
            out[f"dd_{n}"] = dd.copy()
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print("wrote", name)

    # 3. cuboid-restricted steps and interior obstacles (reference semantics
    #    of simulationStepAlpha/Beta(origin, size), src/CLbmSolverGPU.cu:252-337)
    for dtype, tag in ((np.float64, "f64"), (np.float32, "f32")):
        T = np.dtype(dtype).type
        nx, ny, nz = 11, 9, 8
        tau, itau = orc.tau_of(0.032, dtype)
        dd, flags = ref.init(nx, ny, nz, dtype)
        flags[1:-1, ny, 1:-1] = orc.VELOCITY_INJECTION
        flags[3:5, 2:5, 4:7] = orc.OBSTACLE          # a block inside the cavity
        init_flags = flags.copy()
        # z-split into two cuboids each step (as the hybrid split would), plus
        # one partial step restricted to a sub-box
        seq = []
        for i in range(12):
            for (o, s) in (((0, 0, 0), (nx + 2, ny + 2, 4)), ((0, 0, 4), (nx + 2, ny + 2, nz + 2 - 4))):
                seq.append((i & 1, o, s))
        seq.append((0, (2, 1, 3), (5, 6, 4)))
        for kind, o, s in seq:
            if kind:
                ref.beta(dd, flags, itau, T(0.05), origin=o, size=s)
            else:
                ref.alpha(dd, flags, itau, T(0.05), origin=o, size=s)
        np.savez_compressed(os.path.join(HERE, f"cuboid_obstacle_{tag}.npz"),
                            nx=nx, ny=ny, nz=nz, inv_tau=np.array(itau, dtype=dtype),
                            lid_u=np.array(T(0.05), dtype=dtype), flags=init_flags,
                            seq_kind=np.array([k for k, _, _ in seq]),
                            seq_origin=np.array([o for _, o, _ in seq]),
                            seq_size=np.array([s for _, _, s in seq]), dd_final=dd)
        print("wrote cuboid_obstacle", tag)

    if args.skip_digests:
        return
    # 4. digests of larger runs (the 64^3 FP64 case is the CPU-runnable
    #    benchmark configuration, 1000 steps)
    digests = {}
    for name, nx, ny, nz, dtype, nu, U, steps in DIGEST_CASES:
        tau, itau = orc.tau_of(nu, dtype)
        T = np.dtype(dtype).type
        dd, flags = ref.run_cavity(nx, ny, nz, dtype, itau, T(U), steps)
        ux, uy = profiles(dd, last_was_alpha=bool(steps & 1))
        f = post_collision(dd, bool(steps & 1))
        fl = flags[1:-1, 1:-1, 1:-1]
        mask = (fl == orc.FLUID) | (fl == orc.VELOCITY_INJECTION)
        digests[name] = dict(nx=nx, ny=ny, nz=nz, dtype=np.dtype(dtype).name, nu=nu, lid_u=float(T(U)),
                             inv_tau=float(itau), steps=steps, sha256=sha256(dd),
                             mass=float(f[:, mask].sum()), ux_centre=ux.tolist(), uy_centre=uy.tolist())
        print("digest", name, digests[name]["sha256"][:16])
    with open(os.path.join(HERE, "digests.json"), "w") as fh:
        json.dump(digests, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
