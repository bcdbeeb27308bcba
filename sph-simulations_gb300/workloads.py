"""Seeded synthetic initial states for the benchmark configurations.

No dataset is involved: every state is a jittered square lattice built from a
seed.  Physics follows the reference's kernels (poly6 density, spiky pressure,
Laplacian viscosity, linear EOS p = k (rho - rho0)); the parameters each
configuration names that the reference cannot express (rest density 1000,
gravity -9.81, artificial viscosity alpha, periodic boundaries, particle mass)
are the library's extensions.

  dam_break(nx, ny, dx)   water column of nx x ny particles at the left wall of
                          a box (the 12,800- and 1,000,000-particle cases)
  taylor_green(n)         periodic Taylor-Green vortex on [0,1]^2 (512 x 512)
  batch(count)            independent dam-break boxes of log-uniform sizes
                          (256 boxes of 2,000-65,536 particles)
  requests(rate, seconds) a Poisson stream of dam-break / Taylor-Green jobs
                          (200 per second, 1,000-200,000 particles)
  lattice_requests(...)   the same stream as lattice specifications whose
                          initial states the device generates at admission
                          (no host particle arrays: a 60 s window holds
                          12,000 requests, ~450M particles)
"""
import math

import numpy as np

K_STIFF = 30.0   # the reference's GAS_CONSTANT
RHO0 = 1000.0


def poly6_lattice_sum(h, dx):
    """sum_j (h^2 - r_j^2)^3 over a perfect square lattice of spacing dx, r_j <= h."""
    s = 0.0
    m = int(math.ceil(h / dx)) + 1
    for i in range(-m, m + 1):
        for j in range(-m, m + 1):
            r2 = (i * dx) ** 2 + (j * dx) ** 2
            if r2 <= h * h:
                s += (h * h - r2) ** 3
    return s


def lattice_mass(rho0, h, dx):
    """Particle mass that gives rho0 on the perfect lattice with the reference's
    density kernel 315 / (64 pi h^9) (h^2 - r^2)^3."""
    return rho0 / (315.0 / (64.0 * math.pi * h ** 9) * poly6_lattice_sum(h, dx))


def laplacian_lattice_factor(h, dx, mass, rho0):
    """kappa in  sum_j (m/rho) (v_j - v_i) 45/(pi h^6) (h - r)  ~  kappa * lap(v)
    on the lattice, so a kinematic viscosity nu needs MU = nu / kappa."""
    s = 0.0
    m = int(math.ceil(h / dx)) + 1
    for i in range(-m, m + 1):
        for j in range(-m, m + 1):
            r = math.hypot(i * dx, j * dx)
            if 0 < r <= h:
                s += 45.0 / (math.pi * h ** 6) * (h - r) * (i * dx) ** 2
    return 0.5 * (mass / rho0) * s


def _jittered(nx, ny, dx, rng, x0=0.0, y0=0.0):
    gx, gy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = x0 + (gx.ravel() + 0.5) * dx + rng.uniform(-0.01 * dx, 0.01 * dx, gx.size)
    y = y0 + (gy.ravel() + 0.5) * dx + rng.uniform(-0.01 * dx, 0.01 * dx, gx.size)
    return x, y


def dam_break(nx, ny, dx, seed=0, order="morton", box=(1.0, 1.0), alpha=0.1, dt=1e-5):
    """Column of nx x ny particles at the left wall, h = 1.3 dx, walls.

    The reference's laminar viscosity is off (MU = 0): the configurations name
    artificial viscosity alpha as their viscosity, and MU = 0.01 exceeds the
    explicit diffusion limit of dt = 1e-5 at dx = 5e-4."""
    rng = np.random.default_rng(seed)
    x, y = _jittered(nx, ny, dx, rng)
    h = 1.3 * dx
    prm = dict(order=order, h=h, dt=dt, k=K_STIFF, rho0=RHO0, mu=0.0, gx=0.0, gy=-9.81,
               mass=lattice_mass(RHO0, h, dx), alpha=alpha, c0=math.sqrt(K_STIFF),
               lo=(0.0, 0.0), hi=tuple(box), periodic=0)
    z = np.zeros(x.size)
    return prm, x, y, z, z.copy()


def taylor_green(n, seed=0, nu=0.01, order="morton", dt=2e-5):
    """Periodic [0,1]^2, n x n particles, u = sin 2pi x cos 2pi y,
    v = -cos 2pi x sin 2pi y, kinematic viscosity nu, no gravity, no alpha.
    The kinetic energy decays as exp(-16 pi^2 nu t).  Returns (params, x, y,
    vx, vy, ek_rate) with ek_rate = 16 pi^2 nu."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / n
    x, y = _jittered(n, n, dx, rng)
    h = 1.3 * dx
    mass = lattice_mass(RHO0, h, dx)
    kappa = laplacian_lattice_factor(h, dx, mass, RHO0)
    vx = np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    vy = -np.cos(2 * np.pi * x) * np.sin(2 * np.pi * y)
    prm = dict(order=order, h=h, dt=dt, k=K_STIFF, rho0=RHO0, mu=nu / kappa, gx=0.0, gy=0.0,
               mass=mass, alpha=0.0, c0=math.sqrt(K_STIFF), lo=(0.0, 0.0), hi=(1.0, 1.0),
               periodic=1)
    return prm, x, y, vx, vy, 16 * np.pi ** 2 * nu


def dam_break_sized(npart, aspect, dx, rng, alpha, order="morton"):
    """A dam-break instance of about npart particles, column height/width = aspect,
    box 2.5x the column width and 1.25x its height (the proportions of the 12,800-particle case)."""
    nx = max(2, int(round(math.sqrt(npart / aspect))))
    ny = max(2, int(round(npart / nx)))
    x, y = _jittered(nx, ny, dx, rng)
    h = 1.3 * dx
    box = (2.5 * nx * dx, 1.25 * ny * dx)
    prm = dict(order=order, h=h, dt=1e-5, k=K_STIFF, rho0=RHO0, mu=0.0, gx=0.0, gy=-9.81,
               mass=lattice_mass(RHO0, h, dx), alpha=alpha, c0=math.sqrt(K_STIFF),
               lo=(0.0, 0.0), hi=box, periodic=0)
    return prm, x, y


def batch(count=256, seed=0, nmin=2000, nmax=65536, dx=0.005):
    """count independent dam-break boxes: particle counts log-uniform in
    [nmin, nmax], column aspect ratio uniform in [0.3, 2.0], alpha uniform in
    [0.05, 0.2].  Returns (params list, counts, x, y, vx, vy) with the particle
    arrays of all instances concatenated in instance order."""
    rng = np.random.default_rng(seed)
    prms, xs, ys = [], [], []
    for _ in range(count):
        npart = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        aspect = rng.uniform(0.3, 2.0)
        alpha = rng.uniform(0.05, 0.2)
        prm, x, y = dam_break_sized(npart, aspect, dx, rng, alpha)
        prms.append(prm)
        xs.append(x)
        ys.append(y)
    counts = np.array([len(x) for x in xs], np.int64)
    x = np.concatenate(xs)
    y = np.concatenate(ys)
    z = np.zeros(len(x))
    return prms, counts, x, y, z, z.copy()


def requests(rate=200.0, seconds=60.0, seed=0, nmin=1000, nmax=200000, steps=500):
    """Poisson arrivals: list of (arrival_time_s, kind, params, x, y, vx, vy, steps);
    kind is 'dam' or 'tgv' (50/50), particle counts log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        npart = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        if rng.uniform() < 0.5:
            aspect = rng.uniform(0.3, 2.0)
            prm, x, y = dam_break_sized(npart, aspect, 0.005, rng, alpha=0.1)
            vx = np.zeros(len(x))
            vy = np.zeros(len(x))
            out.append((t, "dam", prm, x, y, vx, vy, steps))
        else:
            n = max(8, int(round(math.sqrt(npart))))
            prm, x, y, vx, vy, _ = taylor_green(n, seed=int(rng.integers(1 << 30)))
            out.append((t, "tgv", prm, x, y, vx, vy, steps))
    return out


def lattice_requests(rate=200.0, seconds=60.0, seed=0, nmin=1000, nmax=200000, steps=500):
    """Poisson arrivals as lattice specifications: list of (arrival_time_s, kind,
    params, spec, steps, particles); spec holds the keyword arguments of
    sphg.lattice (x0, y0, dx, dy, nx, ny, jitter, seed, velocity, u0).  kind is
    'dam' (a jittered column at rest, dam_break_sized's geometry) or 'tgv' (the
    periodic Taylor-Green vortex, taylor_green's parameters), 50/50; particle
    counts log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        npart = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        jseed = int(rng.integers(1 << 62))
        if rng.uniform() < 0.5:
            aspect = rng.uniform(0.3, 2.0)
            dx = 0.005
            nx = max(2, int(round(math.sqrt(npart / aspect))))
            ny = max(2, int(round(npart / nx)))
            h = 1.3 * dx
            prm = dict(order="morton", h=h, dt=1e-5, k=K_STIFF, rho0=RHO0, mu=0.0, gx=0.0, gy=-9.81,
                       mass=lattice_mass(RHO0, h, dx), alpha=0.1, c0=math.sqrt(K_STIFF),
                       lo=(0.0, 0.0), hi=(2.5 * nx * dx, 1.25 * ny * dx), periodic=0)
            spec = dict(x0=0.5 * dx, y0=0.5 * dx, dx=dx, dy=dx, nx=nx, ny=ny, jitter=0.01, seed=jseed,
                        velocity=0, u0=0.0)
            out.append((t, "dam", prm, spec, steps, nx * ny))
        else:
            n = max(8, int(round(math.sqrt(npart))))
            dx = 1.0 / n
            h = 1.3 * dx
            mass = lattice_mass(RHO0, h, dx)
            kappa = laplacian_lattice_factor(h, dx, mass, RHO0)
            prm = dict(order="morton", h=h, dt=2e-5, k=K_STIFF, rho0=RHO0, mu=0.01 / kappa, gx=0.0, gy=0.0,
                       mass=mass, alpha=0.0, c0=math.sqrt(K_STIFF), lo=(0.0, 0.0), hi=(1.0, 1.0),
                       periodic=1)
            spec = dict(x0=0.5 * dx, y0=0.5 * dx, dx=dx, dy=dx, nx=n, ny=n, jitter=0.01, seed=jseed,
                        velocity=1, u0=1.0)
            out.append((t, "tgv", prm, spec, steps, n * n))
    return out
