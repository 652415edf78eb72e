"""Seeded synthetic initial conditions for the TreeSPH workloads.

The reference ships no benchmark inputs; these generators produce the five
workload shapes the path is measured on (Plummer sphere, perturbed periodic
lattice, 1/r gas sphere, batched uneven spheres, clustered mixed box).
All positions are FP64.  Every generator takes an explicit seed and uses
numpy's PCG64, so the same call gives the same bytes on any machine.
"""
import math

import numpy as np


def _iso_dirs(rng, n):
    cth = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    sth = np.sqrt(1.0 - cth * cth)
    return np.stack([sth * np.cos(phi), sth * np.sin(phi), cth], axis=1)


def plummer(n, seed=1, a=1.0, mass=1.0, rmax=20.0, G=1.0):
    """Plummer sphere: r = a/sqrt(X^(-2/3)-1) redrawn above rmax*a, speeds by
    Aarseth-Henon-Wielen rejection on g(q) = q^2 (1-q^2)^(7/2)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    r = np.empty(n)
    filled = 0
    while filled < n:
        X = rng.uniform(0.0, 1.0, 2 * (n - filled) + 16)
        X = X[X > 0]
        rr = a / np.sqrt(X ** (-2.0 / 3.0) - 1.0)
        rr = rr[rr <= rmax * a]
        k = min(len(rr), n - filled)
        r[filled:filled + k] = rr[:k]
        filled += k
    pos = _iso_dirs(rng, n) * r[:, None]
    q = np.empty(n)
    filled = 0
    while filled < n:
        m = 4 * (n - filled) + 16
        x1 = rng.uniform(0.0, 1.0, m)
        x2 = rng.uniform(0.0, 0.1, m)
        g = x1 * x1 * (1.0 - x1 * x1) ** 3.5
        acc = x1[x2 < g]
        k = min(len(acc), n - filled)
        q[filled:filled + k] = acc[:k]
        filled += k
    vesc = math.sqrt(2.0 * G * mass / a) * (1.0 + (r / a) ** 2) ** (-0.25)
    vel = _iso_dirs(rng, n) * (q * vesc)[:, None]
    m = np.full(n, mass / n)
    return pos, vel, m


def hernquist(n, seed=1, a=1.0, mass=1.0, rmax=50.0):
    """Hernquist sphere: r = a sqrt(X)/(1-sqrt(X)), clipped at rmax*a; cold
    isotropic velocities at 0.3 of the local circular speed."""
    rng = np.random.Generator(np.random.PCG64(seed))
    r = np.empty(n)
    filled = 0
    while filled < n:
        X = rng.uniform(0.0, 1.0, 2 * (n - filled) + 16)
        sx = np.sqrt(X)
        rr = a * sx / (1.0 - sx)
        rr = rr[(rr <= rmax * a) & np.isfinite(rr)]
        k = min(len(rr), n - filled)
        r[filled:filled + k] = rr[:k]
        filled += k
    pos = _iso_dirs(rng, n) * r[:, None]
    vc = np.sqrt(mass * r / (r + a) ** 2)
    vel = _iso_dirs(rng, n) * (0.3 * vc)[:, None]
    return pos, vel, np.full(n, mass / n)


def _grf_displacement(ng, index, rms, seed, box=1.0):
    """Zel'dovich-style displacement field psi(k) = i k/k^2 delta(k) of a
    Gaussian random field with P(k) ~ k^index on an ng^3 grid, scaled so
    that rms |psi| = rms.  Returns (ng^3, 3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    k1 = np.fft.fftfreq(ng, d=box / ng) * 2.0 * math.pi
    kz1 = np.fft.rfftfreq(ng, d=box / ng) * 2.0 * math.pi
    kx, ky, kz = np.meshgrid(k1, k1, kz1, indexing="ij")
    k2 = kx * kx + ky * ky + kz * kz
    k2[0, 0, 0] = 1.0
    amp = np.sqrt(k2 ** (index / 2.0))
    amp[0, 0, 0] = 0.0
    white = rng.standard_normal((ng, ng, ng))
    delta_k = np.fft.rfftn(white) * amp
    out = np.empty((ng, ng, ng, 3))
    for d, kd in enumerate((kx, ky, kz)):
        psi_k = 1j * kd / k2 * delta_k
        out[..., d] = np.fft.irfftn(psi_k, s=(ng, ng, ng), axes=(0, 1, 2))
    out = out.reshape(-1, 3)
    cur = math.sqrt(float(np.mean(np.sum(out * out, axis=1))))
    return out * (rms / cur)


def lattice_box(ng, seed=2, index=-2.0, rms_frac=0.2, box=1.0, offset=0.0):
    """ng^3 equal-mass particles on a lattice in [-box/2, box/2)^3 displaced
    by a GRF with P(k) ~ k^index, rms displacement rms_frac of the spacing;
    velocities equal to the displacements.  Positions wrapped periodically."""
    dx = box / ng
    g = (np.arange(ng) + 0.5 + offset) * dx - 0.5 * box
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    lat = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    psi = _grf_displacement(ng, index, rms_frac * dx, seed, box)
    pos = lat + psi
    pos = (pos + 0.5 * box) % box - 0.5 * box
    # guard against the modulo landing exactly on +box/2
    pos[pos >= 0.5 * box] -= box
    vel = psi.copy()
    n = ng ** 3
    return pos, vel, np.full(n, 1.0 / n)


def gas_sphere(n, seed=3, R=1.0, mass=1.0, u0=0.05):
    """Evrard-type cold gas sphere: rho ~ 1/r inside R via r = R sqrt(X),
    zero velocity, specific energy u0 G M / R."""
    rng = np.random.Generator(np.random.PCG64(seed))
    X = rng.uniform(0.0, 1.0, n)
    r = R * np.sqrt(X)
    pos = _iso_dirs(rng, n) * r[:, None]
    vel = np.zeros((n, 3))
    u = np.full(n, u0 * mass / R)
    return pos, vel, np.full(n, mass / n), u


def uniform_cube(n, seed=4, box=1.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(-0.5 * box, 0.5 * box, (n, 3))
    return pos, np.zeros((n, 3)), np.full(n, 1.0 / n)


def batched_systems(nsys=512, seed=5, nmin=1024, nmax=65536, gas_frac=0.2):
    """Independent Plummer / Hernquist spheres with N log-uniform in
    [nmin, nmax]; every other system carries a gas fraction.  Returns a
    list of dicts with pos, vel, mass, soft, ngas, a (scale length)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nsys)).astype(np.int64)
    systems = []
    for s in range(nsys):
        n = int(ns[s])
        if s % 2 == 0:
            pos, vel, m = plummer(n, seed=seed * 100003 + s)
        else:
            pos, vel, m = hernquist(n, seed=seed * 100003 + s)
        ngas = int(gas_frac * n) if (s // 2) % 2 == 0 else 0
        systems.append(dict(pos=pos, vel=vel, mass=m, soft=np.full(n, 0.01),
                            ngas=ngas, a=1.0))
    return systems


def pack_systems(systems, u0=0.05):
    """Concatenate independent systems into one particle set for
    Context.set_systems: the gas particles of all systems first (the
    library's convention: gas = the first ngas particles), then the rest.
    Returns (pos, vel, mass, soft, ngas, u, sys_of, index) where index[s] is
    the array of global indices of system s's particles in its own order."""
    gas_idx, dm_idx = [], []
    off = 0
    for s, d in enumerate(systems):
        n = len(d["mass"])
        g = d["ngas"]
        gas_idx.append((s, np.arange(off, off + g)))
        dm_idx.append((s, np.arange(off + g, off + n)))
        off += n
    order = np.concatenate([a for _, a in gas_idx] + [a for _, a in dm_idx])
    sys_cat = np.concatenate([np.full(len(a), s, dtype=np.int32) for s, a in gas_idx] +
                             [np.full(len(a), s, dtype=np.int32) for s, a in dm_idx])
    pos = np.concatenate([d["pos"] for d in systems])[order]
    vel = np.concatenate([d["vel"] for d in systems])[order]
    mass = np.concatenate([d["mass"] for d in systems])[order]
    soft = np.concatenate([d["soft"] for d in systems])[order]
    ngas = int(sum(d["ngas"] for d in systems))
    u = np.full(ngas, u0)
    inv = np.empty(len(order), dtype=np.int64)
    inv[order] = np.arange(len(order))
    index = []
    off = 0
    for d in systems:
        n = len(d["mass"])
        index.append(inv[off:off + n])
        off += n
    return pos, vel, mass, soft, ngas, u, sys_cat, index


def _plummer_offsets(rng, n, a, rmax=20.0):
    """n isotropic offsets with the Plummer radial profile of scale a."""
    r = np.empty(n)
    filled = 0
    while filled < n:
        X = rng.uniform(0.0, 1.0, 2 * (n - filled) + 16)
        X = X[X > 0]
        rr = 1.0 / np.sqrt(X ** (-2.0 / 3.0) - 1.0)
        rr = rr[rr <= rmax]
        k = min(len(rr), n - filled)
        r[filled:filled + k] = rr[:k]
        filled += k
    return _iso_dirs(rng, n) * (r * a)[:, None]


def mixed_box(ng=256, seed=6, index=-1.5, rms_frac=0.3, box=1.0, gas_frac=0.16,
              nclump=64, clump_frac=0.2, amin=0.002, amax=0.02, u0=1e-3):
    """Clustered periodic box of gas and dark matter: two interleaved ng^3
    lattices (gas offset by half a spacing) displaced by one GRF with
    P(k) ~ k^index (rms rms_frac of the spacing), then clump_frac of the
    particles of each species moved into nclump Plummer clumps of scale
    U[amin, amax] at random centres.  Gas holds gas_frac of the mass and
    comes first.  Returns (pos, vel, mass, ngas, u)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dx = box / ng
    psi = _grf_displacement(ng, index, rms_frac * dx, seed, box)
    g = (np.arange(ng) + 0.5) * dx - 0.5 * box
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    lat = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    n = ng ** 3
    gas = lat + 0.5 * dx + psi
    dm = lat + psi
    del lat, X, Y, Z
    pos = np.concatenate([gas, dm])
    del gas, dm
    vel = np.concatenate([psi, psi])
    centres = rng.uniform(-0.5 * box, 0.5 * box, (nclump, 3))
    scales = rng.uniform(amin, amax, nclump)
    for lo in (0, n):                      # each species in turn
        sel = lo + np.nonzero(rng.uniform(0.0, 1.0, n) < clump_frac)[0]
        cid = rng.integers(0, nclump, len(sel))
        off = _plummer_offsets(rng, len(sel), 1.0)
        pos[sel] = centres[cid] + off * scales[cid][:, None]
        vel[sel] = 0.0
    pos = (pos + 0.5 * box) % box - 0.5 * box
    pos[pos >= 0.5 * box] -= box
    mass = np.concatenate([np.full(n, gas_frac / n), np.full(n, (1.0 - gas_frac) / n)])
    return pos, vel, mass, n, np.full(n, u0)
