"""Seeded synthetic particle frames.

There is no public dataset for this pipeline (the reference's sample frames are
an external download), so workloads are generated: a counter-based generator
(splitmix64 finaliser over (seed, stream, index) -> float32 in [0, 1)) makes
every frame bit-identical wherever it is produced.

Frames (sizes follow the reference paper's scenes, restated as synthetic
stand-ins):
* ``water_block``  -- n^3 jittered lattice resting on z >= 0 (plain small case);
* ``crown_splash`` -- jittered pool slab plus a radially launched ring, advected
  ballistically (2M-particle crown splash);
* ``sloshing_tank`` -- frames of an analytic sloshing surface with seeded
  inflow/outflow (batched frames);
* ``dam_break`` -- jittered block over a seeded obstacle, advected by an
  analytic field (8M-particle dam break).
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, count: int, offset: int = 0) -> np.ndarray:
    """float32 uniforms in [0, 1): the top 24 bits of splitmix64(key + i)."""
    with np.errstate(over="ignore"):
        key = np.uint64((seed & 0xFFFFFFFF) << 32) ^ np.uint64((stream & 0xFFFF) << 16)
        idx = np.arange(offset, offset + count, dtype=np.uint64)
        z = _splitmix64((idx * np.uint64(0xD1B54A32D192ED03) + key) & _M64)
    return ((z >> np.uint64(40)).astype(np.float64) * (1.0 / 16777216.0)).astype(np.float32)


def normal(seed: int, stream: int, count: int) -> np.ndarray:
    """Box-Muller normals from two uniform streams (float64 math, float32 out)."""
    u1 = uniform(seed, stream, count).astype(np.float64)
    u2 = uniform(seed, stream + 1, count).astype(np.float64)
    r = np.sqrt(-2.0 * np.log(1.0 - u1))
    return (r * np.cos(2.0 * np.pi * u2)).astype(np.float32)


def lattice(nx: int, ny: int, nz: int, spacing: float, jitter: float, seed: int, origin=(0.0, 0.0, 0.0),
            stream: int = 0) -> np.ndarray:
    """Jittered lattice: p = origin + (i + 0.5) * spacing + U(-jitter, jitter)."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(np.float64)
    base = (base + 0.5) * spacing + np.asarray(origin, np.float64)
    n = base.shape[0]
    jit = (uniform(seed, stream, 3 * n).astype(np.float64).reshape(n, 3) * 2.0 - 1.0) * jitter
    return (base + jit).astype(np.float32)


def water_block(n: int = 64, spacing: float = 0.01, seed: int = 1):
    """Plain small case: n^3 particles, lattice spacing 0.01, jitter +-0.1 spacing,
    block resting on the floor plane z >= 0; zero velocity, rest density 1000."""
    pos = lattice(n, n, n, spacing, 0.1 * spacing, seed)
    vel = np.zeros_like(pos)
    rho = np.full(len(pos), 1000.0, np.float32)
    return pos, vel, rho


def crown_splash(n_slab=(200, 200, 40), spacing: float = 0.005, n_ring: int = 400_000, seed: int = 2,
                 ring_seed: int = 3, t: float = 0.05, radius: float = 0.3, layers: int = 10):
    """2M crown splash: a jittered pool slab plus a seeded crown ring launched
    radially with speed ~ N(1.5, 0.3) m/s, advected ballistically for t seconds
    under gravity -9.81 m/s^2 along z.

    The ring is a cylindrical wall of `layers` radial layers at the lattice
    spacing (SPH particle density, a few particles per cell), centred on the
    slab and standing on its top; its particles fly outward and upward (the
    tilt grows with height, as in a crown), each with its own speed."""
    nx, ny, nz = n_slab
    slab = lattice(nx, ny, nz, spacing, 0.1 * spacing, seed)
    cx, cy = nx * spacing / 2.0, ny * spacing / 2.0
    top = nz * spacing
    # wall lattice: (layer, angle, level) at spacing-sized steps
    rs = radius + spacing * (np.arange(layers) + 0.5)
    per_level = np.maximum(1, np.round(2.0 * np.pi * rs / spacing).astype(np.int64))
    levels = int(np.ceil(n_ring / per_level.sum()))
    lay = np.repeat(np.arange(layers), per_level)
    ang = np.concatenate([np.arange(k) / k for k in per_level]) * 2.0 * np.pi
    lay = np.tile(lay, levels)[:n_ring]
    ang = np.tile(ang, levels)[:n_ring]
    lev = np.repeat(np.arange(levels), per_level.sum())[:n_ring]
    jit = (uniform(ring_seed, 0, 3 * n_ring).astype(np.float64).reshape(-1, 3) * 2.0 - 1.0) * 0.1 * spacing
    r0 = rs[lay] + jit[:, 0]
    theta = ang + jit[:, 1] / rs[lay]
    z0 = top + spacing * (lev + 0.5) + jit[:, 2]
    height = spacing * levels
    speed = 1.5 + 0.3 * normal(ring_seed, 3, n_ring).astype(np.float64)
    tilt = 0.4 + 0.8 * (z0 - top) / height
    dn = np.sqrt(1.0 + tilt * tilt)
    vx, vy, vz = speed * np.cos(theta) / dn, speed * np.sin(theta) / dn, speed * tilt / dn
    x = cx + r0 * np.cos(theta) + vx * t
    y = cy + r0 * np.sin(theta) + vy * t
    z = z0 + vz * t - 0.5 * 9.81 * t * t
    ring = np.stack([x, y, z], 1).astype(np.float32)
    ring_vel = np.stack([vx, vy, vz - 9.81 * t], 1).astype(np.float32)
    pos = np.concatenate([slab, ring])
    vel = np.concatenate([np.zeros_like(slab), ring_vel])
    rho = np.full(len(pos), 1000.0, np.float32)
    return pos, vel, rho


def sloshing_tank(frame: int, n_frames: int = 16, spacing: float = 0.01, length: float = 2.0, width: float = 1.0,
                  depth_min: float = 0.05, depth_max: float = 0.75, amp: float = 0.05, seed: int = 5):
    """Frame k of a sloshing tank: particles fill z <= z0 + A sin(2 pi t) cos(pi x / L),
    t = k / n_frames seconds, with a seeded fill level z0 in [depth_min,
    depth_max] (seeded inflow/outflow), so that at the default sizes the
    particle count varies between about 100k and 1.5M per frame."""
    t = frame / float(n_frames)
    level = uniform(seed + frame, 7, 1)[0]
    z0 = depth_min + (depth_max - depth_min) * level
    nx, ny = int(round(length / spacing)), int(round(width / spacing))
    nz = int(np.ceil((z0 + amp) / spacing)) + 1
    pos = lattice(nx, ny, nz, spacing, 0.1 * spacing, seed + frame)
    surf = z0 + amp * np.sin(2 * np.pi * t) * np.cos(np.pi * pos[:, 0] / length)
    keep = pos[:, 2] <= surf
    pos = pos[keep]
    vz = (amp * 2 * np.pi * np.cos(2 * np.pi * t) * np.cos(np.pi * pos[:, 0] / length)).astype(np.float32)
    vel = np.zeros_like(pos)
    vel[:, 2] = vz * (pos[:, 2] / np.maximum(surf[keep], 1e-6))
    rho = np.full(len(pos), 1000.0, np.float32)
    return pos, vel, rho


def dam_break(shape=(400, 100, 200), spacing: float = 0.005, seed: int = 6, t: float = 0.1):
    """8M dam break: a jittered block over a seeded 0.1-high obstacle, advected
    by an analytic collapse field for t seconds."""
    nx, ny, nz = shape
    pos = lattice(nx, ny, nz, spacing, 0.1 * spacing, seed).astype(np.float64)
    hgt = nz * spacing
    ox = nx * spacing * (1.2 + 0.2 * float(uniform(seed, 9, 1)[0]))
    # collapse: front advances, column sinks (analytic, smooth)
    s = np.clip(pos[:, 2] / hgt, 0, 1)
    vx = 2.0 * np.sqrt(9.81 * hgt) * (1.0 - s) * (pos[:, 0] / (nx * spacing))
    vz = -0.5 * np.sqrt(9.81 * hgt) * s * (pos[:, 0] / (nx * spacing))
    pos[:, 0] += vx * t
    pos[:, 2] += vz * t
    # the obstacle lifts what passes over it
    over = pos[:, 0] > ox
    pos[over, 2] += 0.1 * np.exp(-((pos[over, 0] - ox) / 0.05) ** 2)
    vel = np.stack([vx, np.zeros_like(vx), vz], 1).astype(np.float32)
    rho = np.full(len(pos), 1000.0, np.float32)
    return pos.astype(np.float32), vel, rho


DEFAULT_KEYS = {
    "sim.mass": 1.0,
    "sim.particlespacing": 0.01,
    "surface.smoothingradiusratio": 2,
    "surface.lambdaforsmoothed": 0.0,
    "surface.isovalue": 0.5,
    "surface.isolatenumneighbors": 8,
    "surface.minnumneighbors": 25,
    "diffuse.minkineticenergythreshold": 5.0,
    "diffuse.maxkineticenergythreshold": 50.0,
    "diffuse.mintrappedairthreshold": 5.0,
    "diffuse.maxtrappedairthreshold": 20.0,
    "diffuse.minwavecreststhreshold": 2.0,
    "diffuse.maxwavecreststhreshold": 8.0,
    "diffuse.diffusetrappedairmultiplier": 4000,
    "diffuse.diffusewavecrestsmultiplier": 4000,
    "diffuse.buoyancycontrol": 0.8,
    "diffuse.dragcontrol": 0.5,
    "diffuse.timestep": 0.02,
    "diffuse.lifefimemultiplier": 10,
    "domain.sclargridsizescale": 2,
    "config.gpuid": 0,
    "config.framefrom": 0,
    "config.frameto": 0,
    "config.framestep": 1,
    "config.issurfacereconstruct": "true",
    "config.isdiffusegeneration": "false",
}


# The crown splash workloads (h = 0.01, scalar cell 0.0025).  Diffuse thresholds:
# the reference's sample keys (kinetic energy 5-50, trapped air 5-20) are set for
# its own scenes; with Mass = 1 the ring's kinetic energy 0.5 m |v|^2 is about 1.1
# at 1.5 m/s and its trapped-air potential stays below 4, so both are clamped over
# the ranges the ring covers, and the ring spawns spray, foam and bubbles.
CROWN_KEYS = {
    "sim.particlespacing": 0.005,
    "diffuse.minkineticenergythreshold": 0.5,
    "diffuse.maxkineticenergythreshold": 5.0,
    "diffuse.mintrappedairthreshold": 0.5,
    "diffuse.maxtrappedairthreshold": 4.0,
}


def config_text(**overrides) -> str:
    """config.txt text in the reference's INI layout (bin/config.txt)."""
    keys = dict(DEFAULT_KEYS)
    for k, v in overrides.items():
        keys[k.lower()] = v
    sections: dict[str, list[str]] = {}
    for k, v in keys.items():
        sec, name = k.split(".", 1)
        sections.setdefault(sec, []).append((name, v))
    names = {"sim": "Sim", "surface": "Surface", "diffuse": "Diffuse", "domain": "Domain", "config": "Config"}
    canon = {
        "mass": "Mass", "particlespacing": "ParticleSpacing", "smoothingradiusratio": "SmoothingRadiusRatio",
        "lambdaforsmoothed": "LambdaForSmoothed", "isovalue": "IsoValue", "isolatenumneighbors": "IsolateNumNeighbors",
        "minnumneighbors": "MinNumNeighbors", "minkineticenergythreshold": "MinKineticEnergyThreshold",
        "maxkineticenergythreshold": "MaxKineticEnergyThreshold", "mintrappedairthreshold": "MinTrappedAirThreshold",
        "maxtrappedairthreshold": "MaxTrappedAirThreshold", "minwavecreststhreshold": "MinWaveCrestsThreshold",
        "maxwavecreststhreshold": "MaxWaveCrestsThreshold", "diffusetrappedairmultiplier": "DiffuseTrappedAirMultiplier",
        "diffusewavecrestsmultiplier": "DiffuseWaveCrestsMultiplier", "buoyancycontrol": "BuoyancyControl",
        "dragcontrol": "DragControl", "timestep": "TimeStep", "lifefimemultiplier": "LifefimeMultiplier",
        "sclargridsizescale": "SclarGridSizeScale", "spatialgridsizescale": "SpatialGridSizeScale",
        "gpuid": "GpuId", "framefrom": "Framefrom", "frameto": "Frameto", "framestep": "FrameStep",
        "numzeros": "NumZeros", "issurfacereconstruct": "IsSurfaceReconstruct",
        "isdiffusegeneration": "IsDiffuseGeneration", "fluidpath": "FluidPath", "fluidprefix": "FluidPrefix",
        "surfacepath": "SurfacePath", "surfaceprefix": "SurfacePrefix", "diffusepath": "DiffusePath",
        "diffuseprefix": "DiffusePrefix",
    }
    out = []
    for sec in ("sim", "surface", "diffuse", "domain", "config"):
        if sec not in sections:
            continue
        out.append(f"[{names[sec]}]")
        for name, v in sections[sec]:
            out.append(f"{canon.get(name, name)} = {v}")
        out.append("")
    return "\n".join(out)


def keys_of(**overrides) -> dict:
    keys = dict(DEFAULT_KEYS)
    for k, v in overrides.items():
        keys[k.lower()] = v
    return keys


def crown_variant(seed: int, spacing: float = 0.005, scale: float = 1.0):
    """A seeded crown splash of 1-2M particles (at scale 1): slab footprint,
    depth, ring size, ring radius and flight time drawn from `seed`.  Used as
    training (seeds 100-149) and held-out (seeds 200-209) frames of the
    learned band; `scale` shrinks every particle count for quick runs."""
    u = uniform(seed, 11, 6).astype(np.float64)
    s = scale ** (1.0 / 3.0)
    nx = int(round((170 + 30 * u[0]) * s))
    ny = int(round((170 + 30 * u[1]) * s))
    nz = int(round((30 + 10 * u[2]) * s))
    n_ring = int(round((200_000 + 300_000 * u[3]) * scale))
    radius = (0.18 + 0.12 * u[4]) * s
    t = 0.02 + 0.06 * u[5]
    return crown_splash((nx, ny, nz), spacing, n_ring, seed=seed, ring_seed=seed + 1000, t=t, radius=radius)
