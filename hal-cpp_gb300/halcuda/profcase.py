"""Small, fixed launches of each hot kernel, for ncu captures.

    python -m halcuda.profcase adi 2048 3        # 3 ADI ticks (x-sweep + y-sweep)
    python -m halcuda.profcase explicit 2048 3   # 3 fused explicit ticks
    python -m halcuda.profcase agents 2048 2     # 2 dispatches of 1M agents
    python -m halcuda.profcase stencil64 2048 1  # FP64 per-cell rate diffusion,
                                                 # advection, per-cell advection
    python -m halcuda.profcase wells 0 2         # 2 batched ticks of the 512 wells
    python -m halcuda.profcase adjoint 256 50    # one gradient: 50 steps, checkpoints every 10

Each case builds the benchmark's inputs at the given grid side, runs one
untimed warm-up launch sequence, then the requested number of individually
launched iterations (no CUDA graph), so that `ncu -k <kernel> -c <n>` sees
plain launches with few launches before them.
"""
from __future__ import annotations

import sys

import numpy as np

import halcuda as hal
from halcuda import workloads


def main(argv):
    case = argv[0] if argv else "adi"
    n = int(argv[1]) if len(argv) > 1 else 2048
    iters = int(argv[2]) if len(argv) > 2 else 3
    if case == "adi":
        w = workloads.adi_inputs(n, seed=2, blobs=20)
        with hal.Adi(n, n) as a:
            a.set_field(w["field"])
            a.set_source(w["src"])
            a.profile(1, 5.0, 0.01)
            ms = a.profile(iters, 5.0, 0.01)
        print(f"adi {n}^2: x-sweep {ms[0]*1e3:.1f} us, y-sweep {ms[1]*1e3:.1f} us")
    elif case == "explicit":
        w = workloads.explicit_inputs(n, seed=1)
        with hal.Diffusion(n, n) as d:
            d.set_field(w["field"])
            d.set_point_sources(w["src_idx"], w["src_val"])
            d.profile(1, 0.2, 0.001)
            ms = d.profile(iters, 0.2, 0.001)
        print(f"explicit {n}^2: tick {ms*1e3:.1f} us")
    elif case == "agents":
        agents = max(1, int(1_000_000 * (n / 2048) ** 2))
        w = workloads.agent_inputs(agents, n, seed=3)
        with hal.Agents(n, n, agents) as ag:
            ag.upload(w["positions"], w["radii"])
            ag.profile(1, 1.0, 0.1)
            ms = ag.profile(iters, 1.0, 0.1)
        print(f"agents {agents} in {n}^2: " + ", ".join(f"{v*1e3:.1f}" for v in ms) + " us")
    elif case == "stencil64":
        rng = np.random.default_rng(12)
        cells = n * n
        f, d = rng.random(cells), np.zeros(cells)
        rx, ry = rng.random(cells) * 0.24, rng.random(cells) * 0.24
        vx, vy = rng.random(cells) - 0.5, rng.random(cells) - 0.5
        with hal.Diffusion(n, n) as h:
            for _ in range(iters):
                h.diffuse_var(f, d.copy(), rx, ry, 0, 0)
                h.advect(f, d.copy(), 0.2, -0.1, 0, 0)
                h.advect_var(f, d.copy(), vx, vy, 0, 0)
        print(f"stencil64 {n}^2: {iters} x (diffuse_var, advect, advect_var)")
    elif case == "wells":
        w = workloads.wells_inputs()
        with hal.Wells(w["wells"]) as b:
            for i, f in enumerate(w["fields"]):
                b.set_field(i, f)
            b.set_agents(w["counts"], w["positions"], w["radii"])
            b.run_ticks(1, w["interactionRad"], w["springConstant"])  # autotune + graph capture
            b.sync()
            ms = b.profile(iters, w["interactionRad"], w["springConstant"])
        print("wells: " + ", ".join(f"{v:.3f}" for v in ms) + " ms (explicit, adi x, adi y, agents, tick)")
    elif case == "adjoint":
        rng = np.random.default_rng(4)
        f0 = workloads.gaussian_blobs(n, rng, 8).astype(np.float32)
        D = workloads.rate_field(n, rng).astype(np.float32)
        src = (rng.random(n * n) * 0.01).astype(np.float32)
        with hal.Adjoint(n, n) as a:
            a.set_problem(f0, np.roll(f0, 3), iters, 10)
            a.forward(D, 0.005, src)
            a.gradient(D, 0.005, src)
            t = a.times()
        print(f"adjoint {n}^2, {iters} steps: forward {t[0]:.2f} ms, gradient {t[1]:.2f} ms")
    else:
        raise SystemExit(f"unknown case {case}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
