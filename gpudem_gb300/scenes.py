"""Seeded synthetic scenes: wall meshes and particle beds.

The reference reads its walls from ASCII STL files (TriangleMesh.cu:363) and
places particles by O(N^2) rejection sampling (ParticleSystem.cu:219-285).
Here the same kinds of inputs are generated directly as arrays:

* meshes are ``(T, 3, 3)`` float64 arrays of triangle corners in "file order"
  (the order an STL file would list them), which is what the mesh ingestion
  of the engine (and of the reference loader) consumes;
* particle beds are positions ``(N, 3)`` and radii ``(N,)``, non-overlapping,
  from a seeded ``numpy.random.Generator``.

Gravity points along -y, as in the reference's shipped cases
(demSettings.json "gravity": {"y": -9.81}).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PI_REF_MASS = 3.14      # main.cu:67 uses 3.14 for the sphere volume
PI_REF_DAMP = 3.1415    # ParticleSystem.cu:301 uses 3.1415 in the damping constant


# --------------------------------------------------------------------------- materials

def sphere_mass(rho: float, r):
    """m = rho*3.14*r^3*4/3 in the reference's operation order (main.cu:67)."""
    r = np.asarray(r, dtype=np.float64)
    return (((((rho * PI_REF_MASS) * r) * r) * r) * 4.0) / 3.0


def stiffness_from_E(E: float, r: float) -> float:
    """k = 4/3*(E/2)*sqrt(r/2)*sqrt(0.05 r) (ParticleSystem.cu:202)."""
    return 4.0 / 3.0 * (E * 0.5) * math.sqrt(r * 0.5) * math.sqrt(0.05 * r)


def eta_const(k, e: float):
    """etaconst = -2 ln e sqrt(k/(3.1415^2 + ln^2 e)) (ParticleSystem.cu:301)."""
    k = np.asarray(k, dtype=np.float64)
    le = math.log(e)
    return -2.0 * le * np.sqrt(k / (PI_REF_DAMP * PI_REF_DAMP + le * le))


# --------------------------------------------------------------------------- meshes

def _quad(a, b, c, d):
    """Two triangles (a,b,c) and (a,c,d) of a planar quad, in file order."""
    return [(a, b, c), (a, c, d)]


def box_mesh(half=0.1, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Closed axis-aligned cube of side 2*half: 12 triangles."""
    c = np.asarray(center, dtype=np.float64)
    h = float(half)
    p = lambda x, y, z: tuple(c + h * np.array([x, y, z], dtype=np.float64))
    tris = []
    tris += _quad(p(1, -1, -1), p(1, 1, -1), p(1, 1, 1), p(1, -1, 1))      # +x
    tris += _quad(p(1, -1, 1), p(1, 1, 1), p(-1, 1, 1), p(-1, -1, 1))      # +z
    tris += _quad(p(-1, -1, 1), p(-1, 1, 1), p(-1, 1, -1), p(-1, -1, -1))  # -x
    tris += _quad(p(-1, -1, -1), p(-1, 1, -1), p(1, 1, -1), p(1, -1, -1))  # -z
    tris += _quad(p(-1, 1, -1), p(-1, 1, 1), p(1, 1, 1), p(1, 1, -1))      # +y
    tris += _quad(p(-1, -1, -1), p(1, -1, -1), p(1, -1, 1), p(-1, -1, 1))  # -y
    return np.asarray(tris, dtype=np.float64)


def subdivide(tris: np.ndarray, levels: int) -> np.ndarray:
    """Split every triangle into 4 (midpoint subdivision), `levels` times."""
    t = np.asarray(tris, dtype=np.float64)
    for _ in range(levels):
        a, b, c = t[:, 0], t[:, 1], t[:, 2]
        ab, bc, ca = 0.5 * (a + b), 0.5 * (b + c), 0.5 * (c + a)
        t = np.concatenate([
            np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
            np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)], 0)
    return t


def rotate_z(tris: np.ndarray, deg: float) -> np.ndarray:
    th = math.radians(deg)
    R = np.array([[math.cos(th), -math.sin(th), 0.0],
                  [math.sin(th), math.cos(th), 0.0],
                  [0.0, 0.0, 1.0]])
    return np.einsum("ij,tcj->tci", R, tris)


def tilted_box_mesh(half=0.1, deg=30.0, levels=0) -> np.ndarray:
    """Closed cube tilted by `deg` about z (like geometry/simpleBox30deg.stl),
    optionally face-subdivided (12 * 4**levels triangles)."""
    return rotate_z(subdivide(box_mesh(half), levels), deg)


def helical_chute_mesh(radius=0.3, pitch=0.1, turns=2.0, width=0.12, wall=0.05,
                       n_target=50_000, seed=3, inner_wall=False, end_caps=False,
                       isotropic=False) -> np.ndarray:
    """Parametric helical chute: a ramp winding around the y axis plus an outer
    side wall (and, with `inner_wall`, an inner one; with `end_caps`, walls
    closing both ends), tessellated to about `n_target` triangles.  The ramp
    surface spans radii [radius-width, radius]; the walls stand `wall` high.
    A seeded +-2 % jitter of the ramp's interior radial samples keeps the
    triangles from being perfectly regular."""
    rng = np.random.default_rng(seed)
    n_r = 6                                   # radial quads on the ramp
    n_h = 3                                   # vertical quads on a side wall
    if isotropic:
        # quads about as long as they are wide: side s with
        # (length along the helix) x (ramp width + walls) = (n_target / 2) s^2
        r_mid = radius - 0.5 * width
        length = 2 * math.pi * turns * math.hypot(r_mid, pitch / (2 * math.pi))
        span = width + wall * (2 if inner_wall else 1)
        side = math.sqrt(length * span / (0.5 * n_target))
        n_r = max(1, int(round(width / side)))
        n_h = max(1, int(round(wall / side)))
    per_step = 2 * (n_r + n_h * (2 if inner_wall else 1))
    n_t = max(4, int(round(n_target / per_step)))
    th = np.linspace(0.0, 2 * math.pi * turns, n_t + 1)
    y0 = pitch * th / (2 * math.pi)
    r_in = radius - width
    rr = np.linspace(r_in, radius, n_r + 1)
    jit = 1.0 + 0.02 * (rng.random((n_t + 1, n_r + 1)) - 0.5)
    jit[:, 0] = 1.0
    jit[:, -1] = 1.0
    R = rr[None, :] * jit
    ramp = np.stack([R * np.cos(th)[:, None], np.repeat(-y0[:, None], n_r + 1, 1),
                     R * np.sin(th)[:, None]], -1)            # descends as theta grows
    tris = []
    for a in range(n_t):
        for b in range(n_r):
            tris += _quad(ramp[a, b], ramp[a + 1, b], ramp[a + 1, b + 1], ramp[a, b + 1])
    hh = np.linspace(0.0, wall, n_h + 1)
    wallp = np.stack([radius * np.repeat(np.cos(th)[:, None], n_h + 1, 1),
                      -y0[:, None] + hh[None, :],
                      radius * np.repeat(np.sin(th)[:, None], n_h + 1, 1)], -1)
    for a in range(n_t):
        for b in range(n_h):
            tris += _quad(wallp[a, b], wallp[a + 1, b], wallp[a + 1, b + 1], wallp[a, b + 1])
    if inner_wall:
        innp = np.stack([r_in * np.repeat(np.cos(th)[:, None], n_h + 1, 1),
                         -y0[:, None] + hh[None, :],
                         r_in * np.repeat(np.sin(th)[:, None], n_h + 1, 1)], -1)
        for a in range(n_t):
            for b in range(n_h):
                tris += _quad(innp[a, b], innp[a + 1, b], innp[a + 1, b + 1], innp[a, b + 1])
    if end_caps:
        for a in (0, n_t):
            c, sn = math.cos(th[a]), math.sin(th[a])
            for b in range(n_r):
                for e in range(n_h):
                    r0, r1 = rr[b], rr[b + 1]
                    h0, h1 = -y0[a] + hh[e], -y0[a] + hh[e + 1]
                    tris += _quad(np.array([r0 * c, h0, r0 * sn]), np.array([r1 * c, h0, r1 * sn]),
                                  np.array([r1 * c, h1, r1 * sn]), np.array([r0 * c, h1, r0 * sn]))
    return np.asarray(tris, dtype=np.float64)


def corrugated_floor_mesh(length=1.0, width=0.2, amp=0.003, n_target=200_000, seed=5,
                          periodic=False) -> np.ndarray:
    """Floor of a channel along x with seeded sinusoidal bumps of amplitude
    `amp`, triangulated to about `n_target` triangles (a regular grid of quads)
    over x in [-length/2, length/2], z in [-width/2, width/2].  `periodic`
    rounds the x wavenumber to a whole number of waves per length, so the
    floor continues across x = -length/2 ~ length/2."""
    rng = np.random.default_rng(seed)
    nx = int(math.sqrt(n_target / 2 * length / width))
    nz = max(1, int(n_target / 2 / nx))
    x = np.linspace(-0.5 * length, 0.5 * length, nx + 1)
    z = np.linspace(-0.5 * width, 0.5 * width, nz + 1)
    X, Z = np.meshgrid(x, z, indexing="ij")
    k1, k2 = rng.uniform(20, 60, 2)
    p1, p2 = rng.uniform(0, 2 * math.pi, 2)
    if periodic:
        k1 = 2 * math.pi / length * max(1, round(k1 * length / (2 * math.pi)))
    Y = amp * np.sin(k1 * X + p1) * np.cos(k2 * Z + p2)
    P = np.stack([X, Y, Z], -1)
    a = P[:-1, :-1].reshape(-1, 3)
    b = P[1:, :-1].reshape(-1, 3)
    c = P[1:, 1:].reshape(-1, 3)
    d = P[:-1, 1:].reshape(-1, 3)
    t1 = np.stack([a, b, c], 1)
    t2 = np.stack([a, c, d], 1)
    return np.concatenate([t1, t2], 0)


# --------------------------------------------------------------------------- particles

def random_packing(n, radii, lo, hi, rng, max_trials=2000):
    """Seeded random sequential addition of non-overlapping spheres inside the
    axis-aligned region [lo, hi] (centres kept r away from the faces), with a
    uniform hash grid so it runs in O(N).  Raises if a sphere cannot be placed
    (like ParticleSystem.cu:282)."""
    radii = np.asarray(radii, dtype=np.float64)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    rmax = float(radii.max())
    cell = 2.0 * rmax
    dims = np.maximum(1, np.ceil((hi - lo) / cell).astype(np.int64))
    grid: dict = {}
    pos = np.zeros((n, 3))
    for i in range(n):
        r = radii[i]
        placed = False
        for _ in range(max_trials):
            p = lo + r + rng.random(3) * (hi - lo - 2 * r)
            c = np.minimum(((p - lo) / cell).astype(np.int64), dims - 1)
            ok = True
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        for j in grid.get((c[0] + dx, c[1] + dy, c[2] + dz), ()):
                            d = p - pos[j]
                            if d @ d < (r + radii[j]) ** 2:
                                ok = False
                                break
                        if not ok:
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                pos[i] = p
                grid.setdefault((c[0], c[1], c[2]), []).append(i)
                placed = True
                break
        if not placed:
            raise RuntimeError(f"could not place particle {i} of {n}")
    return pos


def lattice_packing(n, radii, lo, hi, rng, gap=0.1):
    """Jittered simple-cubic lattice fill of [lo, hi] (fast for millions):
    spacing 2*rmax*(1+gap), each centre jittered by up to gap*rmax, so spheres
    never overlap.  Lattice sites are taken in a seeded random order."""
    radii = np.asarray(radii, dtype=np.float64)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    rmax = float(radii.max())
    a = 2.0 * rmax * (1.0 + gap)
    dims = np.floor((hi - lo - 2 * rmax) / a).astype(np.int64) + 1
    total = int(np.prod(dims))
    if total < n:
        raise RuntimeError(f"lattice region holds {total} < {n} spheres")
    sites = rng.permutation(total)[:n]
    iz = sites % dims[2]
    iy = (sites // dims[2]) % dims[1]
    ix = sites // (dims[1] * dims[2])
    base = lo + rmax + np.stack([ix, iy, iz], 1) * a
    jit = (rng.random((n, 3)) - 0.5) * (gap * rmax)
    return base + jit


@dataclass
class Scene:
    """Everything a step engine needs for one scene (SI units, reference layout)."""
    x: np.ndarray            # (N,3) positions
    r: np.ndarray            # (N,)
    m: np.ndarray            # (N,)
    k: np.ndarray            # (N,) normal = tangential stiffness (linear model)
    eta: np.ndarray          # (N,) damping constant (etaconst)
    mu: float
    dt: float
    tris: np.ndarray         # (T,3,3) file-order triangles
    inlet_lo: np.ndarray     # region the box limits must contain (BoundingBox.cu:448)
    inlet_hi: np.ndarray
    g: np.ndarray = field(default_factory=lambda: np.array([0.0, -9.81, 0.0]))
    v: np.ndarray | None = None
    w: np.ndarray | None = None
    skin: float = -1.0       # <= 0 keeps the reference default (r_max)
    refresh: float = -1.0
    # Hertz-Mindlin material (used when the engine runs the HM model)
    E: float = 0.0
    nu: float = 0.0
    e: float = 0.5
    mu_roll: float = 0.0
    name: str = ""
    # contact history in the reference layout (numCont, indHis, deltHis*, and
    # the wall arrays), rows of `hist_stride` slots; None: no contacts yet
    history: dict | None = None
    hist_stride: int = 0
    active: np.ndarray | None = None   # (N,) isActive; None: all active
    # per-particle Hertz-Mindlin friction and restitution (packed scenes)
    mu_p: np.ndarray | None = None
    e_p: np.ndarray | None = None
    # box limits (lo, hi) to use instead of the reference's rule from the mesh
    # and inlet; with periodic_x its x extent is the period
    box: tuple | None = None
    periodic_x: bool = False

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def config1_box_drop(n=100, seed=1) -> Scene:
    """100 monodisperse spheres (r=0.01 m, rho=2500) at seeded non-overlapping
    positions in the upper half of a closed 0.2 m box (12 triangles); linear
    spring-dashpot kn=1e5 N/m, restitution 0.5, mu=0.5, dt=1e-5 s, Verlet
    skin 0.1 r."""
    rng = np.random.default_rng(seed)
    r0 = 0.01
    radii = np.full(n, r0)
    half = 0.1
    x = random_packing(n, radii, [-half, 0.0, -half], [half, half, half], rng)
    m = sphere_mass(2500.0, radii)
    k = np.full(n, 1e5)
    return Scene(x=x, r=radii, m=m, k=k, eta=eta_const(k, 0.5), mu=0.5, dt=1e-5,
                 tris=box_mesh(half), inlet_lo=np.array([-half, 0.0, -half]),
                 inlet_hi=np.array([half, half, half]), skin=0.1 * r0, refresh=0.05 * r0,
                 e=0.5, name="box-drop-100")


def config2_tilted_box(n=30_000, seed=2, r0=2e-3, half=None, levels=0, linear_k=None) -> Scene:
    """Spheres with r ~ U[0.8,1.2]*r0 at seeded random packing in the upper part
    of a closed box tilted 30 degrees (12 triangles).  The Hertz-Mindlin
    material is E=5e6 Pa, nu=0.3, e=0.6, mu=0.4, dt=2e-6 s; `linear_k` (or the
    reference's k(E, r0) law) gives the linear-model twin.  `half` (the box's
    half-width) defaults to 0.1 m, widened in steps of 0.025 m until the
    upper region holds the spheres (0.15 m for 30,000)."""
    rng = np.random.default_rng(seed)
    radii = r0 * rng.uniform(0.8, 1.2, n)
    cs = math.cos(math.radians(30)) + math.sin(math.radians(30))

    def region(h):
        # the tilted cube of half-width h contains the axis-aligned cube of
        # half-width h/(cos30+sin30) around its centre
        s = h / cs
        return np.array([-s, -0.2 * s, -s]), np.array([s, s, s])

    if half is None:
        half = 0.1
        a = 2.0 * radii.max() * 1.05
        while n > 5000 and np.prod(np.floor((region(half)[1] - region(half)[0] - 2 * radii.max()) / a) + 1) < n:
            half += 0.025
    lo, hi = region(half)
    x = lattice_packing(n, radii, lo, hi, rng, gap=0.05) if n > 5000 else \
        random_packing(n, radii, lo, hi, rng)
    m = sphere_mass(2500.0, radii)
    kk = stiffness_from_E(5e6, r0) if linear_k is None else linear_k
    k = np.full(n, kk)
    return Scene(x=x, r=radii, m=m, k=k, eta=eta_const(k, 0.6), mu=0.4, dt=2e-6,
                 tris=tilted_box_mesh(half, 30.0, levels), inlet_lo=lo, inlet_hi=hi,
                 E=5e6, nu=0.3, e=0.6, name=f"tilted-box-{n}")


def lognormal_radii(n, rng, median=1e-3, sigma=0.15, lo=0.6e-3, hi=1.6e-3):
    r = median * np.exp(sigma * rng.standard_normal(n))
    return np.clip(r, lo, hi)


def config3_helical_chute(n=1_000_000, seed=3, n_tri=50_000, radius=0.3, pitch=0.1, width=0.12,
                          v_sigma=0.0) -> Scene:
    """1e6 lognormal spheres (median 1 mm, sigma_log 0.15, clipped [0.6,1.6] mm)
    over a seeded helical chute (radius 0.3 m, pitch 0.1 m, 2 turns, ~5e4
    triangles).  The spheres start on a jittered lattice filling the annulus
    above the ramp (radii [radius-width, radius]) from just above the ramp's
    highest point upwards, in a seeded random order of lattice sites.  HM
    material E=5e6 Pa, nu=0.3, e=0.5, mu=0.5; dt=1e-6 s.  `v_sigma` adds
    seeded Gaussian initial velocities (m/s)."""
    rng = np.random.default_rng(seed)
    radii = lognormal_radii(n, rng)
    tris = helical_chute_mesh(radius=radius, pitch=pitch, width=width, n_target=n_tri, seed=seed)
    rmax = float(radii.max())
    a = 2.0 * rmax * 1.05
    r_in, r_out = radius - width + rmax + 1e-3, radius - rmax - 1e-3
    xs = np.arange(-r_out, r_out + 1e-12, a)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    rr = np.hypot(X, Z)
    keep = (rr >= r_in) & (rr <= r_out)
    cols = np.stack([X[keep], Z[keep]], 1)
    layers = int(math.ceil(n / cols.shape[0]))
    y0 = 0.01 + rmax
    sites = rng.permutation(cols.shape[0] * layers)[:n]
    col = sites % cols.shape[0]
    lay = sites // cols.shape[0]
    x = np.stack([cols[col, 0], y0 + lay * a, cols[col, 1]], 1)
    x += (rng.random((n, 3)) - 0.5) * (0.05 * rmax)
    lo = x.min(0) - rmax
    hi = x.max(0) + rmax
    m = sphere_mass(2500.0, radii)
    k = np.full(n, stiffness_from_E(5e6, 1e-3))
    v = rng.normal(0.0, v_sigma, (n, 3)) if v_sigma > 0 else None
    return Scene(x=x, r=radii, m=m, k=k, eta=eta_const(k, 0.5), mu=0.5, dt=1e-6,
                 tris=tris, inlet_lo=lo, inlet_hi=hi, v=v, E=5e6, nu=0.3, e=0.5,
                 name=f"helical-chute-{n}")


def config3_chute_pour(n=1_000_000, seed=3, n_tri=50_000, radius=0.3, pitch=0.1, width=0.12, turns=3.0,
                       wall=0.09) -> Scene:
    """The poured-chute inlet state: 1e6 lognormal spheres (median 1 mm,
    sigma_log 0.15, clipped [0.6,1.6] mm) on a jittered loose lattice resting
    just above every turn of a closed helical chute (radius 0.3 m, pitch
    0.1 m, 3 turns, inner and outer walls 9 cm high, end walls, ~5e4
    triangles of about 7 mm), filled from the ramp upwards, at rest.  HM material E=5e6 Pa,
    nu=0.3, e=0.5, mu=0.5; dt=1e-6 s.  `settle_scene` pours it into a bed."""
    rng = np.random.default_rng(seed)
    radii = lognormal_radii(n, rng)
    tris = helical_chute_mesh(radius=radius, pitch=pitch, turns=turns, width=width, wall=wall,
                              n_target=n_tri, seed=seed, inner_wall=True, end_caps=True, isotropic=True)
    rmax = float(radii.max())
    a = 2.0 * rmax * 1.02
    r_in, r_out = radius - width + rmax + 2e-3, radius - rmax - 2e-3
    xs = np.arange(-r_out, r_out + 1e-12, a)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    rr = np.hypot(X, Z)
    keep = (rr >= r_in) & (rr <= r_out)
    cols = np.stack([X[keep], Z[keep]], 1)
    th = np.mod(np.arctan2(cols[:, 1], cols[:, 0]), 2 * math.pi)
    n_turns = int(turns)
    per_layer = cols.shape[0] * n_turns
    layers = int(math.ceil(n / per_layer))
    if (layers - 1) * a + 2 * rmax + 2e-3 > pitch - 2 * rmax:
        raise ValueError("the lattice does not fit between the chute's turns")
    site = np.arange(per_layer * layers)
    lay = site // per_layer
    rest = site % per_layer
    turn = rest // cols.shape[0]
    col = rest % cols.shape[0]
    # fill the lowest layers first, in a seeded order within the top layer
    order = np.lexsort((rng.random(site.size), lay))[:n]
    lay, turn, col = lay[order], turn[order], col[order]
    ramp_y = -pitch * (th[col] + 2 * math.pi * turn) / (2 * math.pi)
    x = np.stack([cols[col, 0], ramp_y + rmax + 1e-3 + lay * a, cols[col, 1]], 1)
    x += (rng.random((n, 3)) - 0.5) * (0.05 * rmax)
    perm = rng.permutation(n)              # pId order unrelated to position
    x = x[perm]
    lo = x.min(0) - rmax
    hi = x.max(0) + rmax
    m = sphere_mass(2500.0, radii)
    k = np.full(n, stiffness_from_E(5e6, 1e-3))
    return Scene(x=x, r=radii, m=m, k=k, eta=eta_const(k, 0.5), mu=0.5, dt=1e-6,
                 tris=tris, inlet_lo=lo, inlet_hi=hi, E=5e6, nu=0.3, e=0.5,
                 name=f"helical-chute-pour-{n}")


def settle_scene(sc: Scene, steps=10_000, dt=2e-5, e=0.1, precision="mixed", hist_stride=32,
                 chunk=1000, log=None) -> Scene:
    """Pour `sc` into a bed on the GPU: run the engine (Hertz-Mindlin) with a
    larger time step `dt` and restitution `e` for `steps` steps, then return
    the scene at that state (positions, velocities, spins, tangential
    history) with the original time step and material.  Deterministic for a
    given scene and GPU."""
    from dataclasses import replace
    from .engine import Engine
    pour = replace(sc, dt=dt, e=e, history=None, hist_stride=0)
    E = Engine(pour, precision=precision, model="hertz_mindlin", hist_capacity=hist_stride,
               hist_wall_capacity=min(hist_stride, 16))
    done = 0
    while done < steps:
        c = min(chunk, steps - done)
        E.step(c)
        done += c
        if log is not None:
            st = E.stats()
            log(f"settle step {done}: active {st['n_active']} KE {st['kinetic_energy']:.3e} "
                f"contacts/particle {st['coordination']:.2f} rebuilds {st['rebuilds']} error {st['error_word']}")
    st = E.export(history=True, hist_stride=hist_stride)
    E.close()
    hist = {k: st[k] for k in ("numCont", "indHis", "deltHisx", "deltHisy", "deltHisz", "numContWall",
                               "indHisWall", "deltHisxWall", "deltHisyWall", "deltHiszWall")}
    act = st["isActive"] == 1
    return replace(sc, x=st["x"].reshape(-1, 3), v=st["v"].reshape(-1, 3), w=st["angv"].reshape(-1, 3),
                   history=hist, hist_stride=hist_stride, active=act,
                   name=sc.name + f"-settled{steps}")


def box_mesh_grid(half=0.1, k=1, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Closed axis-aligned cube of side 2*half with every face split into k x k
    quads: 12 k^2 triangles."""
    c = np.asarray(center, dtype=np.float64)
    h = float(half)
    faces = [  # corner, u axis, v axis (outward normal = u x v)
        ((1, -1, -1), (0, 2, 0), (0, 0, 2)), ((-1, -1, 1), (2, 0, 0), (0, 2, 0)),
        ((-1, -1, -1), (0, 0, 2), (0, 2, 0)), ((-1, -1, -1), (0, 2, 0), (2, 0, 0)),
        ((-1, 1, -1), (0, 0, 2), (2, 0, 0)), ((-1, -1, -1), (2, 0, 0), (0, 0, 2)),
    ]
    tris = []
    for o, u, w in faces:
        o, u, w = (np.asarray(a, dtype=np.float64) for a in (o, u, w))
        for i in range(k):
            for j in range(k):
                p = lambda a, b: c + h * (o + u * (a / k) + w * (b / k))
                tris += _quad(p(i, j), p(i + 1, j), p(i + 1, j + 1), p(i, j + 1))
    return np.asarray(tris, dtype=np.float64)


def config4_batched(n_scenes=256, seed=4, n_min=1000, n_max=50_000) -> list:
    """Batched ensemble: `n_scenes` independent box-drop scenes.  Each has a
    particle count log-uniform in [n_min, n_max], radii uniform in
    [0.9, 1.1] mm, its own closed box tilted 30 degrees (12 k^2 triangles, k in
    1..13, so 12 to 2,028), sized so its spheres start on a loose lattice in
    the middle, and its own friction mu in [0.2, 0.7] and restitution e in
    [0.3, 0.9].  Hertz-Mindlin, E = 5e6 Pa, nu = 0.3, dt = 1e-6 s."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        radii = rng.uniform(0.9e-3, 1.1e-3, n)
        rmax = float(radii.max())
        a = 2.0 * rmax * 1.05
        per_axis = math.ceil(n ** (1.0 / 3.0)) + 1
        half = (per_axis * a + 2 * rmax) / 0.9          # lattice region = middle 90 % of the half-size
        k = int(rng.integers(1, 14))
        tris = rotate_z(box_mesh_grid(half, k), 30.0)
        lo = np.full(3, -0.45 * half)
        hi = np.full(3, 0.45 * half)
        x = lattice_packing(n, radii, lo, hi, rng, gap=0.05)
        m = sphere_mass(2500.0, radii)
        kk = np.full(n, stiffness_from_E(5e6, 1e-3))
        mu = float(rng.uniform(0.2, 0.7))
        e = float(rng.uniform(0.3, 0.9))
        out.append(Scene(x=x, r=radii, m=m, k=kk, eta=eta_const(kk, e), mu=mu, dt=1e-6, tris=tris,
                         inlet_lo=lo, inlet_hi=hi, E=5e6, nu=0.3, e=e, name=f"batch-{s}-{n}"))
    return out


def pack_scenes(scenes: list, gap=None):
    """Independent scenes side by side in one domain, for one engine: their
    bounding boxes (mesh and spheres) shelf-packed `gap` apart (default eight
    maximum radii, well beyond the Verlet cutoff, so no two scenes ever list
    each other), every scene translated by its offset.  Returns the packed
    Scene, with per-particle friction and restitution, and the offsets (S, 3)
    and particle ranges (S + 1,)."""
    rmax = max(float(np.max(sc.r)) for sc in scenes)
    gap = 8.0 * rmax if gap is None else gap
    lo = [np.minimum(sc.tris.reshape(-1, 3).min(0), np.asarray(sc.x).min(0) - rmax) for sc in scenes]
    hi = [np.maximum(sc.tris.reshape(-1, 3).max(0), np.asarray(sc.x).max(0) + rmax) for sc in scenes]
    ext = [h - l + gap for l, h in zip(lo, hi)]
    width = 1.3 * sum(float(np.prod(e)) for e in ext) ** (1.0 / 3.0)
    order = sorted(range(len(scenes)), key=lambda s: -float(np.max(ext[s])))
    offs = np.zeros((len(scenes), 3))
    x0 = z0 = y0 = 0.0
    row_d = layer_h = 0.0
    for s in order:
        e = ext[s]
        if x0 + e[0] > width and x0 > 0:
            x0, z0 = 0.0, z0 + row_d
            row_d = 0.0
        if z0 + e[2] > width and z0 > 0:
            x0, z0, y0 = 0.0, 0.0, y0 + layer_h
            row_d = layer_h = 0.0
        offs[s] = np.array([x0, y0, z0]) - lo[s]
        x0 += e[0]
        row_d = max(row_d, e[2])
        layer_h = max(layer_h, e[1])
    cat = lambda f: np.concatenate([f(s, sc) for s, sc in enumerate(scenes)], 0)
    x = cat(lambda s, sc: np.asarray(sc.x) + offs[s])
    tris = cat(lambda s, sc: np.asarray(sc.tris) + offs[s])
    zeros3 = lambda sc: np.zeros((sc.n, 3))
    v = cat(lambda s, sc: np.asarray(sc.v) if sc.v is not None else zeros3(sc))
    w = cat(lambda s, sc: np.asarray(sc.w) if sc.w is not None else zeros3(sc))
    starts = np.concatenate([[0], np.cumsum([sc.n for sc in scenes])])
    first = scenes[0]
    packed = Scene(x=x, r=cat(lambda s, sc: sc.r), m=cat(lambda s, sc: sc.m), k=cat(lambda s, sc: sc.k),
                   eta=cat(lambda s, sc: sc.eta), mu=first.mu, dt=first.dt, tris=tris,
                   inlet_lo=x.min(0) - rmax, inlet_hi=x.max(0) + rmax, g=first.g, v=v, w=w,
                   E=first.E, nu=first.nu, e=first.e, mu_roll=first.mu_roll,
                   mu_p=cat(lambda s, sc: np.full(sc.n, sc.mu)), e_p=cat(lambda s, sc: np.full(sc.n, sc.e)),
                   name=f"packed-{len(scenes)}-scenes")
    return packed, offs, starts


def side_wall_mesh(length, z, y0, y1, pieces=8) -> np.ndarray:
    """Vertical wall z = const over x in [-length/2, length/2], y in [y0, y1],
    as `pieces` quads along x (two triangles each)."""
    xs = np.linspace(-0.5 * length, 0.5 * length, pieces + 1)
    tris = []
    for a, b in zip(xs[:-1], xs[1:]):
        tris += _quad(np.array([a, y0, z]), np.array([b, y0, z]), np.array([b, y1, z]), np.array([a, y1, z]))
    return np.asarray(tris, np.float64)


def config5_periodic_channel(n=10_000_000, seed=5, length=1.0, width=0.5, n_tri=200_000, amp=0.003,
                             v_drift=0.0, v_sigma=0.1, dt=1e-6) -> Scene:
    """Spheres in a channel periodic in x: bidisperse radii 1.0 / 1.5 mm at
    70 / 30 (seeded), a floor of about `n_tri` triangles with seeded
    sinusoidal corrugation of amplitude `amp` (a whole number of waves per
    period), flat side walls at z = +-width/2 cut into pieces narrower than a
    quarter period, open top.  The spheres start on a jittered lattice above
    the floor with seeded Gaussian velocities (`v_sigma`) plus `v_drift` along
    x.  Hertz-Mindlin E=5e6 Pa, nu=0.3, e=0.5, mu=0.5, rolling friction 0.05.
    The box's x extent [-length/2, length/2) is the period."""
    rng = np.random.default_rng(seed)
    radii = np.where(rng.random(n) < 0.7, 1.0e-3, 1.5e-3)
    rmax = float(radii.max())
    floor = corrugated_floor_mesh(length, width, amp, n_tri - 32, seed, periodic=True)
    a = 2.0 * rmax * 1.05
    nxl = int(math.floor(length / a))
    nzl = int(math.floor((width - 2 * rmax - 2e-3) / a))
    per_layer = nxl * nzl
    layers = int(math.ceil(n / per_layer))
    y_top = amp + 2e-3 + rmax + layers * a
    walls = np.concatenate([side_wall_mesh(length, -0.5 * width, -amp - 0.01, y_top + 0.01),
                            side_wall_mesh(length, 0.5 * width, -amp - 0.01, y_top + 0.01)])
    tris = np.concatenate([floor, walls])
    sites = rng.permutation(per_layer * layers)[:n]
    ix = sites % nxl
    iz = (sites // nxl) % nzl
    iy = sites // per_layer
    x = np.stack([-0.5 * length + (ix + 0.5) * (length / nxl),
                  amp + 2e-3 + rmax + iy * a,
                  -0.5 * width + rmax + 1e-3 + (iz + 0.5) * a], 1)
    x += (rng.random((n, 3)) - 0.5) * (0.04 * rmax)
    m = sphere_mass(2500.0, radii)
    k = np.full(n, stiffness_from_E(5e6, 1e-3))
    v = rng.normal(0.0, v_sigma, (n, 3)) if v_sigma > 0 else np.zeros((n, 3))
    v[:, 0] += v_drift
    lo = np.array([-0.5 * length, -amp - 0.02, -0.5 * width - 0.01])
    hi = np.array([0.5 * length, y_top + 0.05, 0.5 * width + 0.01])
    return Scene(x=x, r=radii, m=m, k=k, eta=eta_const(k, 0.5), mu=0.5, dt=dt, tris=tris,
                 inlet_lo=lo, inlet_hi=hi, v=v, E=5e6, nu=0.3, e=0.5, mu_roll=0.05,
                 box=(lo, hi), periodic_x=True, name=f"periodic-channel-{n}")


# --------------------------------------------------------------------------- physics checks
# Small scenes for the reference's physics-level comparisons: the LIGGGHTS
# two-sphere collision (liggghtsCases/testCases/in.collision) and the analytic
# scripts python/compareDrop.py, compareRoll.py and compareCollision.py.

def hooke_stiffness(Y: float, nu: float, r1: float, r2: float, m1: float, m2: float, v_char: float) -> float:
    """Normal stiffness of LIGGGHTS' `hooke` pair model (its documented
    formula): kn = 16/15 sqrt(R*) Y* (15 m* V^2 / (16 sqrt(R*) Y*))^(1/5) with
    Y* = 1/((1-nu^2)/Y + (1-nu^2)/Y), R* = r1 r2/(r1+r2), m* = m1 m2/(m1+m2) and
    V the characteristic velocity.  LIGGGHTS uses the same value tangentially."""
    ystar = 1.0 / (2.0 * (1.0 - nu * nu) / Y)
    rstar = r1 * r2 / (r1 + r2)
    mstar = m1 * m2 / (m1 + m2)
    sq = math.sqrt(rstar)
    return 16.0 / 15.0 * sq * ystar * (15.0 * mstar * v_char * v_char / (16.0 * sq * ystar)) ** 0.2


def hooke_eta_const(kn: float, e: float) -> float:
    """etaconst for which the linear law's damping etaconst * sqrt(m*) equals
    LIGGGHTS' hooke gamma_n = sqrt(4 m* kn / (1 + (pi / ln e)^2)), i.e. the
    reference's formula (ParticleSystem.cu:301) with pi in full."""
    le = math.log(e)
    return -2.0 * le * math.sqrt(kn / (math.pi * math.pi + le * le))


def two_sphere_scene(x, v, r, m, k, eta, mu: float, dt: float, half: float = 1.0) -> Scene:
    """Two spheres without walls or gravity in the cube [-half, half]^3, with
    the linear law's per-sphere k and etaconst."""
    n = len(r)
    return Scene(x=np.asarray(x, np.float64).reshape(n, 3), r=np.asarray(r, np.float64),
                 m=np.asarray(m, np.float64), k=np.asarray(k, np.float64), eta=np.asarray(eta, np.float64),
                 mu=mu, dt=dt, tris=np.zeros((0, 3, 3)), inlet_lo=np.full(3, -half),
                 inlet_hi=np.full(3, half), g=np.zeros(3), v=np.asarray(v, np.float64).reshape(n, 3),
                 w=np.zeros((n, 3)), name="two-spheres")


def bouncing_sphere_scene(y0=0.5, floor=-1.0, r=0.01, rho=1000.0, k=1e5, e=0.3, mu=0.5, dt=5e-6) -> Scene:
    """python/compareDrop.py's case: one sphere released at rest at height y0
    above a horizontal floor (two triangles at y = floor), gravity -9.81 y."""
    m = sphere_mass(rho, np.full(1, r))
    kk = np.full(1, k)
    a, b = 0.1, floor
    tris = np.asarray(_quad(np.array([-a, b, -a]), np.array([-a, b, a]), np.array([a, b, a]),
                            np.array([a, b, -a])), np.float64)
    return Scene(x=np.array([[0.0, y0, 0.0]]), r=np.full(1, r), m=m, k=kk, eta=eta_const(kk, e), mu=mu, dt=dt,
                 tris=tris, inlet_lo=np.array([-a, floor, -a]), inlet_hi=np.array([a, y0 + 2 * r, a]),
                 v=np.zeros((1, 3)), w=np.zeros((1, 3)), e=e, name="bouncing-sphere")


def incline_scene(theta_deg=60.0, mu=0.2, r=0.01, rho=1000.0, k=1e5, e=0.3, dt=1e-5, length=0.6) -> Scene:
    """python/compareRoll.py's case: one sphere at rest on a plane inclined by
    theta, descending along d = (cos theta, -sin theta, 0), touching at the
    static overlap m g cos(theta) / k.  It slides with a = g (sin - mu cos)
    when mu < 2/7 tan(theta) and rolls with a = 5/7 g sin otherwise."""
    th = math.radians(theta_deg)
    d = np.array([math.cos(th), -math.sin(th), 0.0])
    nrm = np.array([math.sin(th), math.cos(th), 0.0])
    z = np.array([0.0, 0.0, 1.0])
    w = 0.05
    tris = np.asarray(_quad(-0.05 * d - w * z, -0.05 * d + w * z, length * d + w * z, length * d - w * z), np.float64)
    m = sphere_mass(rho, np.full(1, r))
    kk = np.full(1, k)
    x0 = (r - float(m[0]) * 9.81 * math.cos(th) / k) * nrm
    v = tris.reshape(-1, 3)
    return Scene(x=x0[None, :], r=np.full(1, r), m=m, k=kk, eta=eta_const(kk, e), mu=mu, dt=dt, tris=tris,
                 inlet_lo=v.min(0) - 2 * r, inlet_hi=v.max(0) + 2 * r, v=np.zeros((1, 3)), w=np.zeros((1, 3)),
                 e=e, name="incline")
