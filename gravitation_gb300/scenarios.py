"""Seeded synthetic scenarios (host, numpy, FP64).

The reference only ships an unseeded ``galaxy`` generator (gravitation/lib/simulation.py:
99-184, ``random.random``) and a two-body solar system (simulation.py:85-97).  The
workloads measured here are seeded instead, so that every run sees the same bodies:

  uniform_cube   positions U[-1000,1000]^3, velocities N(0,1)^3, masses U[1,100]
  plummer_pair   two Plummer spheres, sampled by the method of Aarseth, Henon and
                 Wielen (1974, A&A 37, 183), masses log-uniform
  batch_sizes / batch_universes   many universes of log-uniform size
  galaxy         the reference's galaxy recipe (simulation.py:99-184) on a seeded
                 generator

All values are in the universe's (scaled) units: they are what ``add_object`` stores
after scaling (_base_.py:114-117).
"""

import math

import numpy as np

G_DEFAULT = 6.6740831e-11   # universe_base default (_base_.py:73)
T_DEFAULT = 1.0e3           # universe_base default (_base_.py:72)


def uniform_cube(n, seed=0, half=1000.0, v_sigma=1.0, m_lo=1.0, m_hi=100.0):
    """(r[n,3], v[n,3], m[n]) with r ~ U[-half,half]^3, v ~ N(0, v_sigma), m ~ U[m_lo,m_hi]."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(-half, half, (n, 3))
    v = rng.normal(0.0, v_sigma, (n, 3))
    m = rng.uniform(m_lo, m_hi, n)
    return r, v, m


def _isotropic(rng, n, radius):
    z = (1.0 - 2.0 * rng.random(n)) * radius
    phi = 2.0 * math.pi * rng.random(n)
    rho = np.sqrt(np.maximum(radius * radius - z * z, 0.0))
    return np.stack([rho * np.cos(phi), rho * np.sin(phi), z], axis=1)


def plummer_sphere(rng, n, a, m, G):
    """One Plummer sphere of scale radius `a` and masses `m` (centred, at rest).

    Aarseth, Henon & Wielen (1974): the radius follows from inverting the cumulative
    mass M(r)/M = r^3 / (r^2 + a^2)^(3/2); the speed is q times the local escape
    speed, with q drawn by rejection from g(q) ~ q^2 (1 - q^2)^(7/2).
    """
    mtot = float(m.sum())
    x = rng.uniform(1e-10, 0.999, n)  # cut the far tail at 99.9% of the mass
    r = a / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
    pos = _isotropic(rng, n, r)
    q = np.empty(n)
    filled = 0
    while filled < n:
        k = 2 * (n - filled) + 16
        x4 = rng.random(k)
        x5 = rng.random(k)
        ok = 0.1 * x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
        take = x4[ok][: n - filled]
        q[filled:filled + take.size] = take
        filled += take.size
    vesc = math.sqrt(2.0 * G * mtot / a) * (1.0 + (r / a) ** 2) ** -0.25
    vel = _isotropic(rng, n, q * vesc)
    pos -= (m[:, None] * pos).sum(axis=0) / mtot
    vel -= (m[:, None] * vel).sum(axis=0) / mtot
    return pos, vel


def plummer_pair(n, seed=2, a=50.0, sep=1000.0, vrel=5.0, m_lo=0.1, m_hi=1000.0, G=G_DEFAULT):
    """Two Plummer spheres of n//2 bodies (the first gets the odd one), centres at
    (-sep/2, 0, 0) and (+sep/2, 0, 0), approaching with relative speed `vrel` along x;
    masses log-uniform in [m_lo, m_hi]."""
    rng = np.random.default_rng(seed)
    m = np.exp(rng.uniform(math.log(m_lo), math.log(m_hi), n))
    n1 = n - n // 2
    parts = []
    for idx, (cx, vx) in enumerate(((-0.5 * sep, 0.5 * vrel), (0.5 * sep, -0.5 * vrel))):
        sl = slice(0, n1) if idx == 0 else slice(n1, n)
        p, v = plummer_sphere(rng, sl.stop - sl.start, a, m[sl], G)
        p[:, 0] += cx
        v[:, 0] += vx
        parts.append((p, v))
    r = np.concatenate([parts[0][0], parts[1][0]])
    v = np.concatenate([parts[0][1], parts[1][1]])
    return r, v, m


def batch_sizes(n_univ=256, seed=1, n_min=64, n_max=16384):
    """Universe sizes drawn log-uniform in [n_min, n_max]."""
    rng = np.random.default_rng(seed)
    s = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_univ))
    return np.clip(np.rint(s).astype(np.int64), n_min, n_max)


def batch_universes(n_univ=256, seed=1, n_min=64, n_max=16384):
    """Sizes plus one uniform_cube per universe (seed derived from (seed, u))."""
    sizes = batch_sizes(n_univ, seed, n_min, n_max)
    out = []
    for u, n in enumerate(sizes):
        ss = int(np.random.SeedSequence([seed, u]).generate_state(1)[0])
        out.append(uniform_cube(int(n), seed=ss))
    return sizes, out


def mass_perturbation(n, seed, lo=0.99, hi=1.01):
    """Seeded per-body mass factors in [lo, hi] (the adjoint workload's target run)."""
    return np.random.default_rng(np.random.SeedSequence([seed, 7])).uniform(lo, hi, n)


def galaxy(n, seed=0, G=G_DEFAULT, scale_r=1.0e-10, scale_m=1.0e-30, m_hole=4e40,
           m_star=2e30, radius=1e20):
    """The reference's galaxy scenario (simulation.py:57-77, 99-184) with a seeded
    generator: one central black hole plus n-1 stars on circular orbits, 4/5 in a thin
    disc and 1/5 in a central bulge.  Returns unscaled SI values (r, v, m) and the
    universe parameters (T, scale_m, scale_r) the reference uses for it."""
    rng = np.random.default_rng(seed)
    Gs = G * scale_r ** 3 / scale_m  # _base_.py:85-88
    stars = n - 1
    r = np.zeros((n, 3))
    v = np.zeros((n, 3))
    m = np.full(n, m_star)
    m[0] = m_hole
    span = 4.6 * radius
    for k in range(stars):
        alpha = rng.random() * 2.0 * math.pi
        if k < stars * 4 // 5:
            r_abs = (rng.random() * 4.5 + 0.1) * radius
            pos = [r_abs * math.cos(alpha), r_abs * math.sin(alpha),
                   (0.5 * rng.random() - 0.25) * radius * (span - r_abs) / span]
        else:
            r_abs = (rng.random() * 0.75 + 0.1) * radius
            beta = math.pi * (rng.random() - 0.5)
            pos = [r_abs * math.cos(alpha) * math.cos(beta),
                   r_abs * math.sin(alpha) * math.cos(beta), r_abs * math.sin(beta)]
        # circular speed around the hole with the universe's scaled G and SI values,
        # as simulation.py:147-149 does (the rotations by zero angles are omitted)
        v_abs = math.sqrt(Gs * m_hole / math.sqrt(sum(c * c for c in pos)))
        va = alpha - 0.5 * math.pi
        r[k + 1] = pos
        v[k + 1] = [v_abs * math.cos(va), v_abs * math.sin(va), 0.0]
    return r, v, m, dict(T=2.0e12, scale_m=scale_m, scale_r=scale_r, dtype='float32')
