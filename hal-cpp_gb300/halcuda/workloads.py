"""Seeded synthetic inputs for the benchmark workloads.

numpy's PCG64 stands in for Hal::Rand (xoshiro256**); the shapes, sizes and
value distributions are the workloads' own:

* explicit   -- field U[0,1); 64 distinct point sources of 0.05; Dirichlet 1.0
                on the x = -1 edge, 0.0 elsewhere; rate 0.2; decay 0.001
* adi        -- sum of 200 Gaussian blobs (centre U[0,n)^2, sigma 10 + U[0,70),
                amplitude U[0,1)); constant source field U[0,0.01); rate 5.0;
                decay 0.01; zero-flux
* agents     -- 70% uniform and 30% in a Gaussian cluster (sigma 100 cells)
                at a seeded centre, clamped into the domain; float32
                positions; radius 0.5; cutoff 1.0; stiffness 0.1; walls
* wells      -- 512 independent square wells, side round(64 * 16^U) (log-
                uniform in [64, 1024]); half explicit with rate U[0.05, 0.24],
                half ADI with rate U[1, 10]; decay U[0, 0.02]; field U[0,1);
                0..20000 uniform agents each (radius 0.5, cutoff 1.0,
                stiffness 0.1, walls)
* adjoint    -- 512 x 512, 500 steps, zero-flux; rate field D(x) = 0.5 + 4.5 *
                normalise(sum of 32 cosine modes, integer wave numbers in
                [-4, 4], N(0,1) amplitudes, U[0, 2pi) phases); decay 0.005;
                source U[0, 0.01); initial field 40 Gaussian blobs; target =
                the final field of the same model with a second seeded D
"""
from __future__ import annotations

import numpy as np


def explicit_inputs(n: int = 256, seed: int = 1, n_sources: int = 64):
    rng = np.random.default_rng(seed)
    field = rng.random(n * n)
    sites = rng.choice(n * n, n_sources, replace=False).astype(np.int32)
    values = np.full(n_sources, 0.05)
    ghost = np.zeros(4 * n)
    ghost[:n] = 1.0  # bc(-1, y) = 1.0
    return dict(field=field, src_idx=sites, src_val=values, ghost=ghost, diffRate=0.2,
                decay=0.001, xDim=n, yDim=n)


def gaussian_blobs(n: int, rng, count: int = 200):
    field = np.zeros((n, n))
    coord = np.arange(n, dtype=np.float64)
    for _ in range(count):
        cx, cy = rng.random(2) * n
        sigma = 10.0 + rng.random() * 70.0
        amp = rng.random()
        ex = np.exp(-((coord - cx) ** 2) / (2.0 * sigma * sigma))
        ey = np.exp(-((coord - cy) ** 2) / (2.0 * sigma * sigma))
        field += amp * np.outer(ex, ey)
    return field.ravel()


def adi_inputs(n: int = 2048, seed: int = 2, blobs: int = 200):
    rng = np.random.default_rng(seed)
    field = gaussian_blobs(n, rng, blobs)
    src = rng.random(n * n) * 0.01
    return dict(field=field, src=src, diffRate=5.0, decay=0.01, xDim=n, yDim=n)


def agent_inputs(n_agents: int = 1_000_000, dim: int = 2048, seed: int = 3):
    rng = np.random.default_rng(seed)
    m = int(round(n_agents * 0.3))
    uni = rng.random((n_agents - m, 2)) * dim
    centre = rng.random(2) * dim
    clu = centre + rng.normal(0.0, 100.0, (m, 2))
    pos = np.concatenate([uni, clu])
    hi = np.nextafter(np.float32(dim), np.float32(0))
    pos = np.clip(pos, 0.0, float(hi)).astype(np.float32)
    radii = np.full(n_agents, 0.5, dtype=np.float32)
    return dict(positions=pos.ravel(), radii=radii, interactionRad=1.0, springConstant=0.1,
                xDim=dim, yDim=dim, uptake=0.001)


def wells_inputs(n_wells: int = 512, seed: int = 4, max_agents: int = 20000, min_side: int = 64,
                 max_side: int = 1024):
    """Well descriptors (hal.Wells dicts) plus per-well fields and agents."""
    rng = np.random.default_rng(seed)
    ratio = max_side / min_side
    sides = np.rint(min_side * ratio ** rng.random(n_wells)).astype(np.int32)
    kinds = rng.random(n_wells) < 0.5
    wells, fields, counts, pos, rad = [], [], [], [], []
    for i in range(n_wells):
        n = int(sides[i])
        adi = bool(kinds[i])
        rate = float(rng.uniform(1.0, 10.0) if adi else rng.uniform(0.05, 0.24))
        decay = float(rng.uniform(0.0, 0.02))
        na = int(rng.integers(0, max_agents + 1))
        wells.append(dict(xDim=n, yDim=n, kind="adi" if adi else "explicit", diffRate=rate, decay=decay,
                          maxAgents=na))
        fields.append(rng.random(n * n).astype(np.float32))
        counts.append(na)
        hi = np.nextafter(np.float32(n), np.float32(0))
        pos.append(np.minimum(rng.random(2 * na) * n, hi).astype(np.float32))
        rad.append(np.full(na, 0.5, dtype=np.float32))
    return dict(wells=wells, fields=fields, counts=np.array(counts, dtype=np.int32),
                positions=np.concatenate(pos) if pos else np.zeros(0, np.float32),
                radii=np.concatenate(rad) if rad else np.zeros(0, np.float32),
                interactionRad=1.0, springConstant=0.1)


def rate_field(n: int, rng, modes: int = 32, lo: float = 0.5, hi: float = 5.0):
    """Smooth random rate field in [lo, hi] from `modes` cosine modes."""
    x = np.arange(n, dtype=np.float64)
    X, Y = np.meshgrid(x, x, indexing="ij")
    acc = np.zeros((n, n))
    for _ in range(modes):
        kx, ky = rng.integers(-4, 5, 2)
        amp = rng.standard_normal()
        phase = rng.random() * 2.0 * np.pi
        acc += amp * np.cos(2.0 * np.pi * (kx * X + ky * Y) / n + phase)
    span = acc.max() - acc.min()
    acc = (acc - acc.min()) / (span if span > 0 else 1.0)
    return (lo + (hi - lo) * acc).ravel()


def adjoint_inputs(n: int = 512, seed: int = 5, steps: int = 500):
    """Parameter-recovery problem: initial field, the unknown rate field D, a
    second seeded ground-truth rate field, decay and source."""
    rng = np.random.default_rng(seed)
    f0 = gaussian_blobs(n, rng, 40)
    D = rate_field(n, rng)
    D_true = rate_field(n, rng)
    src = rng.random(n * n) * 0.01
    return dict(f0=f0.astype(np.float32), D=D.astype(np.float32), D_true=D_true.astype(np.float32),
                src=src.astype(np.float32), decay=0.005, steps=steps, checkpoint_every=22, xDim=n, yDim=n,
                fd_directions=64, fd_h=1e-3)
