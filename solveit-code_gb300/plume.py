"""Seeded synthetic electrospray plumes (the workloads' input generator).

A plume is a cylinder of singly charged ions: radius 20 nm, length L along z,
positions uniform in the cylinder, species 50/50 monomer (EMI+, 111 amu,
species code 0) and dimer ((EMI)2BF4+, 309 amu, code 1), axial velocity
N(2e4, 2e3) m/s, transverse N(0, 500) m/s, all inbound and injected at t=0.
The species codes, masses and status values are those of the reference's
ParticleSpecies / ParticleStatus enums (structures.h:206-221, particles.h:65-87).

Seeds follow seed = 1000*workload + realisation with numpy's PCG64, so every
test, fixture and benchmark draws the same particles for the same workload.
"""
from __future__ import annotations

import numpy as np

MONOMER_AMU = 111.0
DIMER_AMU = 309.0

# name -> (N, plume length in metres)
WORKLOADS = {
    "direct_n4096": (4096, 1e-6),
    "bh_n65536": (65536, 10e-6),
    "fmm_n1m": (1 << 20, 50e-6),
    "adjoint_n16384": (16384, 1e-6),
}


def make_plume(n: int, length: float, seed: int, radius: float = 20e-9,
               vz_mean: float = 2e4, vz_std: float = 2e3, vt_std: float = 500.0):
    """Return a dict of float64 state arrays for n ions.

    x, v: (n, 3) metres and m/s; q: charge in e; m: mass in amu;
    species: int32 code; status: int32 (1 = inbound); t_inj: seconds.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    r = radius * np.sqrt(rng.random(n))
    phi = 2.0 * np.pi * rng.random(n)
    z = length * rng.random(n)
    species = (rng.random(n) < 0.5).astype(np.int32)
    vz = rng.normal(vz_mean, vz_std, n)
    vx = rng.normal(0.0, vt_std, n)
    vy = rng.normal(0.0, vt_std, n)
    x = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    v = np.stack([vx, vy, vz], axis=1)
    m = np.where(species == 1, DIMER_AMU, MONOMER_AMU)
    return {
        "x": np.ascontiguousarray(x, dtype=np.float64),
        "v": np.ascontiguousarray(v, dtype=np.float64),
        "q": np.ones(n, dtype=np.float64),
        "m": m.astype(np.float64),
        "species": species,
        "status": np.ones(n, dtype=np.int32),
        "t_inj": np.zeros(n, dtype=np.float64),
    }


def make_ball(n: int, radius: float, seed: int):
    """make_plume's ions (species, velocities) placed uniformly in a ball of
    the given radius about the origin: a plume resolved in all three
    dimensions, as a batch's plumes become once they expand."""
    st = make_plume(n, 1e-6, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    r = radius * rng.random(n) ** (1.0 / 3.0)
    st["x"] = np.ascontiguousarray(u * r[:, None])
    return st


def make_batch(nplumes: int = 256, config: int = 3, nmin: int = 1024, nmax: int = 65536,
               length: float = 1e-6, direct_below: int = 8192):
    """The batched-plume workload: nplumes independent realisations.

    Plume sizes are uniform integers in [nmin, nmax] drawn with seed
    1000*config + 999; plume i is make_plume(N_i, length, 1000*config + i).
    Plumes with N < direct_below use the direct sum, the others the FMM; the
    even-numbered plumes use the 4-fold rotational variant.
    Returns (states, methods, symmetries) with method 0 = direct, 2 = FMM and
    symmetry 0 = none, 1 = rotational (the C ABI's codes).
    """
    rng = np.random.Generator(np.random.PCG64(1000 * config + 999))
    sizes = rng.integers(nmin, nmax + 1, size=nplumes)
    states = [make_plume(int(n), length, 1000 * config + i) for i, n in enumerate(sizes)]
    methods = [0 if int(n) < direct_below else 2 for n in sizes]
    syms = [1 if i % 2 == 0 else 0 for i in range(nplumes)]
    return states, methods, syms


def concat(states):
    """One state dict holding every plume back to back, and the plume sizes."""
    keys = ("x", "v", "q", "m", "species", "status", "t_inj")
    out = {k: np.ascontiguousarray(np.concatenate([s[k] for s in states])) for k in keys}
    return out, np.array([s["x"].shape[0] for s in states], np.int64)


def to_ref32(state):
    """Pack a plume into the reference's FP32 vec4 arrays.

    position = (x, y, z, q), velocity = (vx, vy, vz, species),
    acceleration = (0, 0, 0, status), plus timeInjected (particles.h:99-105).
    """
    n = state["x"].shape[0]
    pos4 = np.zeros((n, 4), np.float32)
    vel4 = np.zeros((n, 4), np.float32)
    acc4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = state["x"]
    pos4[:, 3] = state["q"]
    vel4[:, :3] = state["v"]
    vel4[:, 3] = state["species"]
    acc4[:, 3] = state["status"]
    t_inj = state["t_inj"].astype(np.float32)
    return pos4, vel4, acc4, t_inj


def from_ref32(pos4, vel4, acc4, t_inj=None):
    """Widen the reference's FP32 vec4 arrays into FP64 state arrays."""
    n = pos4.shape[0]
    species = vel4[:, 3].astype(np.int32)
    return {
        "x": pos4[:, :3].astype(np.float64),
        "v": vel4[:, :3].astype(np.float64),
        "q": pos4[:, 3].astype(np.float64),
        "m": np.where(species == 1, DIMER_AMU, MONOMER_AMU).astype(np.float64),
        "species": species,
        "status": acc4[:, 3].astype(np.int32),
        "t_inj": (np.zeros(n) if t_inj is None else t_inj.astype(np.float64)),
    }
