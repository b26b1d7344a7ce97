"""Seeded synthetic BAT trajectories of a linear chain.

The reference takes bond/angle/torsion (BAT) trajectories from MD; no
trajectory ships with it, so workloads are generated with the shapes and
value distributions below and a fixed seed:

* a chain of ``A`` atoms has ``A-1`` bonds, ``A-2`` angles, ``A-3`` torsions;
* bonds ~ Normal(1.5 A, 0.03), angles ~ Normal(1.91 rad, 0.08);
* torsions ~ von Mises mixture, modes (-pi/3, pi/3, pi), kappa 8, weights
  0.4/0.3/0.3.  A latent mode index couples torsions: with ``coupling=
  "neighbour"`` torsion t copies torsion t-1's mode with probability 0.7;
  with ``coupling="block8"`` each torsion takes the mode of its block of 8
  consecutive torsions with probability 0.7, else draws its own;
* values are stored as float32 (the reference reads BAT with
  ``nc_get_vara_float``, src/Netcdf_BAT.cpp:247) and torsions are wrapped to
  [0, 2*pi) (the reference's torsion binning assumes non-negative angles,
  src/Real2Int.cpp:459-476).

Arrays are DOF-major ``[ndof][nframes]``, the reference's in-memory layout
after ``Netcdf_BAT::readMulti*Frames`` (src/Netcdf_BAT.cpp:236-330).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

TWO_PI = 2.0 * np.pi
MODES = np.array([-np.pi / 3.0, np.pi / 3.0, np.pi])
WEIGHTS = np.array([0.4, 0.3, 0.3])


@dataclass
class BATTrajectory:
    bonds: np.ndarray      # [nbond][nframes] float32
    angles: np.ndarray     # [nangle][nframes] float32
    torsions: np.ndarray   # [ntors][nframes] float32 in [0, 2pi)

    @property
    def nframes(self) -> int:
        return int(self.bonds.shape[1])

    @property
    def ndof(self) -> int:
        return len(self.bonds) + len(self.angles) + len(self.torsions)

    def blocks(self):
        return ((1, self.bonds), (2, self.angles), (3, self.torsions))


def chain_trajectory(natoms: int, nframes: int, seed: int = 0,
                     coupling: str = "neighbour", kappa: float = 8.0,
                     p_share: float = 0.7) -> BATTrajectory:
    if natoms < 4:
        raise ValueError("a chain needs at least 4 atoms")
    rng = np.random.default_rng(seed)
    nb, na, nt = natoms - 1, natoms - 2, natoms - 3
    bonds = rng.normal(1.5, 0.03, size=(nb, nframes)).astype(np.float32)
    angles = rng.normal(1.91, 0.08, size=(na, nframes)).astype(np.float32)
    # angles must stay inside (0, pi); the tails of N(1.91, 0.08) never reach
    # the bounds at these sizes, the clip only guards against that
    np.clip(angles, np.float32(1e-3), np.float32(np.pi - 1e-3), out=angles)

    cum = np.cumsum(WEIGHTS)
    modes = np.empty((nt, nframes), np.int8)

    def draw(size):
        return np.searchsorted(cum, rng.random(size), side="right").astype(np.int8)

    if coupling == "neighbour":
        modes[0] = draw(nframes)
        for t in range(1, nt):
            fresh = draw(nframes)
            keep = rng.random(nframes) < p_share
            modes[t] = np.where(keep, modes[t - 1], fresh)
    elif coupling == "block8":
        for b0 in range(0, nt, 8):
            b1 = min(nt, b0 + 8)
            latent = draw(nframes)
            for t in range(b0, b1):
                fresh = draw(nframes)
                keep = rng.random(nframes) < p_share
                modes[t] = np.where(keep, latent, fresh)
    else:
        raise ValueError(f"unknown coupling {coupling!r}")
    noise = rng.vonmises(0.0, kappa, size=(nt, nframes))
    tors = np.mod(MODES[modes] + noise, TWO_PI).astype(np.float32)
    # float32 rounding can land exactly on 2*pi; keep the half-open range
    tors[tors >= np.float32(TWO_PI)] = np.float32(0.0)
    return BATTrajectory(bonds, angles, tors)


# Named workloads (chain size, frames, bins, steps, coupling).
WORKLOADS = {
    "chain25": dict(natoms=25, nframes=50_000, nbins=30, nsteps=4, coupling="neighbour"),
    "chain200": dict(natoms=200, nframes=100_000, nbins=50, nsteps=10, coupling="block8"),
    "chain1000": dict(natoms=1000, nframes=100_000, nbins=50, nsteps=10, coupling="block8"),
    "chain5000": dict(natoms=5000, nframes=100_000, nbins=50, nsteps=10, coupling="block8"),
}

# Batched trajectories of uneven size: 16 chains of 200..1200 atoms with
# 20,000..150,000 frames (sizes and lengths paired by a seeded permutation),
# 40 bins, 10 convergence steps.
BATCHES = {
    "batch16": dict(nsys=16, atoms=(200, 1200), frames=(20_000, 150_000), nbins=40, nsteps=10,
                    coupling="block8"),
    "batch4": dict(nsys=4, atoms=(40, 120), frames=(5_000, 30_000), nbins=40, nsteps=10,
                   coupling="block8"),
}


def batch_specs(name: str, seed: int = 0):
    """(natoms, nframes, seed) of every trajectory of a named batch."""
    b = BATCHES[name]
    n = b["nsys"]
    atoms = np.linspace(b["atoms"][0], b["atoms"][1], n).round().astype(int)
    frames = np.linspace(b["frames"][0], b["frames"][1], n).round().astype(int)
    frames = frames[np.random.default_rng(seed).permutation(n)]
    return [(int(a), int(f), seed * 1000 + k) for k, (a, f) in enumerate(zip(atoms, frames))]


def _vonmises_torch(torch, shape, kappa, gen, device):
    """Von Mises(0, kappa) samples by the Best-Fisher (1979) rejection method."""
    tau = 1.0 + np.sqrt(1.0 + 4.0 * kappa * kappa)
    rho = (tau - np.sqrt(2.0 * tau)) / (2.0 * kappa)
    r = (1.0 + rho * rho) / (2.0 * rho)
    out = torch.empty(shape, dtype=torch.float64, device=device).view(-1)
    todo = torch.arange(out.numel(), device=device)
    while todo.numel():
        m = todo.numel()
        u = torch.rand((3, m), generator=gen, device=device, dtype=torch.float64)
        z = torch.cos(np.pi * u[0])
        f = (1.0 + r * z) / (r + z)
        c = kappa * (r - f)
        ok = (c * (2.0 - c) - u[1] > 0) | (torch.log(c / u[1]) + 1.0 - c >= 0)
        th = torch.sign(u[2] - 0.5) * torch.acos(f.clamp(-1.0, 1.0))
        out[todo[ok]] = th[ok]
        todo = todo[~ok]
    return out.view(shape)


def chain_blocks_torch(natoms: int, nframes: int, seed: int, device, coupling: str = "block8",
                       kappa: float = 8.0, p_share: float = 0.7):
    """The chain of ``chain_trajectory`` (same distributions and coupling)
    drawn on a device with torch, for workloads too large to generate on
    the host: [(bat_type, float32 tensor [k][nframes])] for bonds, angles,
    torsions."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    nb, na, nt = natoms - 1, natoms - 2, natoms - 3
    bonds = (torch.randn((nb, nframes), generator=gen, device=device) * 0.03 + 1.5).float()
    angles = (torch.randn((na, nframes), generator=gen, device=device) * 0.08 + 1.91)
    angles = angles.clamp(1e-3, np.pi - 1e-3).float()
    cum = torch.tensor(np.cumsum(WEIGHTS), device=device)
    modes_v = torch.tensor(MODES, device=device)

    def draw(size):
        u = torch.rand(size, generator=gen, device=device, dtype=torch.float64)
        return torch.searchsorted(cum, u, right=True).clamp(max=len(WEIGHTS) - 1)

    tors = torch.empty((nt, nframes), dtype=torch.float32, device=device)
    step = 8 if coupling == "block8" else nt
    prev = None
    for b0 in range(0, nt, step):
        b1 = min(nt, b0 + step)
        k = b1 - b0
        fresh = draw((k, nframes))
        keep = torch.rand((k, nframes), generator=gen, device=device) < p_share
        if coupling == "block8":
            latent = draw((1, nframes)).expand(k, nframes)
            modes = torch.where(keep, latent, fresh)
        else:
            modes = fresh.clone()
            for t in range(k):
                src = prev if t == 0 else modes[t - 1]
                if src is not None:
                    modes[t] = torch.where(keep[t], src, fresh[t])
            prev = modes[-1]
        ang = modes_v[modes] + _vonmises_torch(torch, (k, nframes), kappa, gen, device)
        ang = torch.remainder(ang, TWO_PI).float()
        ang[ang >= np.float32(TWO_PI)] = 0.0
        tors[b0:b1] = ang
    return [(1, bonds), (2, angles), (3, tors)]
