"""Seeded synthetic scenes with the shapes of the benchmark configurations.

No public dataset is involved: every scene is a cubic particle lattice with uniform
jitter, inside triangulated walls, built from a seed.

  dam_break      - 0.8 x 0.2 x 0.6 m box (12-triangle STL), fluid column
                   0.2 x 0.2 x 0.4 m at l0 = 0.01 (16,000 particles)
  rotating_bucket - closed cylinder r = 0.15 m, L = 0.3 m, 4096 triangles, axis
                   horizontal along x, 35 % filled, 30 rpm, optional drag spheres
                   (icospheres of radius 3*l0); l0 = 0.004 gives ~116k particles,
                   l0 = 0.002 ~0.93M
  mixer          - four such buckets of seeded radius 0.10-0.18 m, 40 % filled,
                   20-45 rpm, one shared grid

Particle and wall parameters follow the reference's parameter file fields
(CParameter); lambda for the reference schedule comes from its l0 table
(MultiGPUHandler.cpp:757-921) and the physics schedule uses lattice values.
"""
from dataclasses import dataclass, field
import math
from typing import List, Optional

import numpy as np

from .types import (CParameter, CTriangleParameters, DragParameter, CGridBox, Scalar3, grid_box)


@dataclass
class Scene:
    name: str
    param: CParameter
    box: CGridBox
    pos: np.ndarray            # (N,3) float64
    vel: np.ndarray            # (N,3) float64
    press: np.ndarray          # (N,)  float64
    visc: np.ndarray           # (N,)  float64
    ptype: np.ndarray          # (N,)  int32
    tri_vertices: np.ndarray   # (T,3,3) float64
    tri_model: np.ndarray      # (T,)  int32
    tri_params: List[CTriangleParameters] = field(default_factory=list)
    drag: List[DragParameter] = field(default_factory=list)
    n0_pnd: float = 0.0        # lattice PND at re_grad
    n0_lap: float = 0.0        # lattice PND at re_lap
    lam: float = 0.0           # lattice Laplacian lambda

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    @property
    def t(self) -> int:
        return int(self.tri_vertices.shape[0])


def lattice_constants(re_coef: float, l0: float = 1.0, dim: int = 3):
    """n0 = sum of w(r) = re/r - 1 and lambda = sum r^2 w / sum w over the cubic
    lattice points within re (the centre excluded), in FP64."""
    m = int(math.ceil(re_coef)) + 1
    rng = np.arange(-m, m + 1, dtype=np.float64)
    if dim == 3:
        g = np.stack(np.meshgrid(rng, rng, rng, indexing="ij"), -1).reshape(-1, 3)
    else:
        g = np.stack(np.meshgrid(rng, rng, indexing="ij"), -1).reshape(-1, 2)
    r = np.sqrt((g ** 2).sum(-1))
    msk = (r > 0) & (r < re_coef)
    w = re_coef / r[msk] - 1.0
    n0 = float(w.sum())
    lam = float((r[msk] ** 2 * w).sum() / w.sum()) * l0 * l0
    return n0, lam


def lambda_table(l0: float) -> float:
    """The reference's lambda(l0) fit (CalculateLambdaValueLocal, MultiGPUHandler.cpp:
    757-921) including its chained-comparison branch selection: the first row whose
    lower bound is not below l0 (l0 as float, promoted), or the first row with an
    upper bound >= 1, is taken.  Evaluated as a*l0 + b in float."""
    rows = [(0, 0.0001, 5.02608E-06, 3.82946E-10), (0.0001, 0.0005, 0.000124918, 1.81984E-08),
            (0.0005, 0.001, 0.0017886, -4.84707E-07), (0.001, 0.002, 0.00373277, -2.15486E-06),
            (0.002, 0.003, 0.0066746, -6.72384E-06), (0.003, 0.004, 0.0107452, -1.76386E-05),
            (0.004, 0.005, 0.0141993, -3.08052E-05), (0.005, 0.006, 0.0164975, -4.14937E-05),
            (0.006, 0.007, 0.0181782, -4.95251E-05), (0.007, 0.008, 0.0205885, -6.28759E-05),
            (0.008, 0.009, 0.0222761, -7.17244E-05), (0.009, 0.01, 0.0231972, -7.34117E-05),
            (0.01, 0.02, 0.0369119, -0.000210081), (0.02, 0.03, 0.0667457, -0.000672376),
            (0.03, 0.04, 0.106105, -0.00171939), (0.04, 0.05, 0.141998, -0.00308074),
            (0.05, 0.06, 0.164981, -0.00414971), (0.05, 0.06, 0.164981, -0.00414971),
            (0.06, 0.07, 0.178483, -0.00474469), (0.07, 0.08, 0.197539, -0.00567825),
            (0.08, 0.09, 0.208407, -0.00598107), (0.09, 0.1, 0.211437, -0.00543137),
            (0.01, 0.5, 0.369118, -0.021008), (0.5, 1, 1.78861, -0.48471),
            (1, 10, 0.423015, 4.1213), (10, 1000, 0.0138964, 745.762)]
    f = np.float32
    l0f = f(l0)
    a = b = f(0)
    for lo, hi, ra, rb in rows:
        lt = 1.0 if lo < float(l0f) else 0.0
        if lt <= hi:
            a, b = f(ra), f(rb)
            break
    return float(f(a * l0f) + b)


def default_param(l0: float, dt: float, *, explicit_pressure: bool = False, sonic: float = 20.0,
                  courant: float = 0.2, quirk_lambda: bool = True) -> CParameter:
    p = CParameter()
    p.Dimension = 3
    p.GravityConstant = Scalar3(0.0, 0.0, -9.81)
    p.Density = 1000.0
    n0g, _ = lattice_constants(2.1)
    p.ConstantParticleDensity = n0g
    p.InitialParticleDistance = l0
    p.FreeSurfaceThreshold = 0.97
    p.GradientInfluenceRadiusCoefficient = 2.1
    p.LaplacianInfluenceRadiusCoefficient = 4.0
    p.TemperatureInfluenceRadiusCoefficient = 2.1
    p.FruidSpecificHeat = 4186.0
    p.FruidDensity = 1000.0
    p.Dt = dt
    p.AnalysisStep = 1000
    p.ThermalStep = 1
    p.OutputStep = 100
    p.CourantNumber = courant
    p.OffSet = 0.5
    p.WallFrictionCoeffieicnt = 1.0
    p.StopWallStep = 2 ** 31 - 1
    p.Tolerance = 0.0
    p.bExplicitPressure = explicit_pressure
    p.SonicVelocity = sonic
    p.ArtificialPressure = 0.0
    p.r_coeff = 0.0
    p.PressureMax = 3.4e38
    p.RLimitCoefficient = 3.4e38
    p.ConstantCheckStep = -1
    p.MaxNeighborhoodNum = 729
    p.LambdaValue = lambda_table(l0) if quirk_lambda else lattice_constants(4.0, l0)[1]
    return p


def _tri_normal_params(model_velocity=(0, 0, 0), rotating=False, rpm=0.0, dt=1e-4, center=(0, 0, 0),
                       second=(1, 0, 0), start=0.0, reach=0.0, is_drag=False, drag_id=0,
                       friction=1.0) -> CTriangleParameters:
    tp = CTriangleParameters()
    tp.Velocity = Scalar3(*model_velocity)
    tp.RotatingOrNot = rotating
    # per-step angle, as MultiGPUHandler.cpp:485 computes it (RPM is an Integer there)
    tp.AngleOfRotationInDegree = float(np.float32(int(rpm)) * np.float32(dt) * np.float32(6)) if rotating else 0.0
    tp.RotationInRPM = float(int(rpm))
    tp.RotationStartTime = start
    tp.TimeToReachRPM = reach
    tp.CenterOfRotation = Scalar3(*center)
    tp.SecondPointOfRotation = Scalar3(*second)
    tp.WallFrictionCoefficient = friction
    tp.isDrag = is_drag
    tp.DragTriangleID = drag_id
    tp.LinearResetInterval = 1
    return tp


def box_triangles(lo, hi) -> np.ndarray:
    """12 triangles of an axis-aligned box, normals pointing inward."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float64)
    faces = [(0, 1, 2), (0, 2, 3),      # bottom z0, normal +z
             (4, 6, 5), (4, 7, 6),      # top z1, normal -z
             (0, 4, 5), (0, 5, 1),      # y0, normal +y
             (3, 2, 6), (3, 6, 7),      # y1, normal -y
             (0, 3, 7), (0, 7, 4),      # x0, normal +x
             (1, 5, 6), (1, 6, 2)]      # x1, normal -x
    return np.array([[v[a], v[b], v[c]] for a, b, c in faces])


def cylinder_triangles(center, radius, length, n_theta=64, n_len=31) -> np.ndarray:
    """Closed cylinder along x: n_theta*n_len*2 side triangles + 2*n_theta cap
    triangles (64*31*2 + 128 = 4096), normals pointing inward."""
    cx, cy, cz = center
    th = np.linspace(0.0, 2 * np.pi, n_theta + 1)[:-1]
    xs = np.linspace(cx - length / 2, cx + length / 2, n_len + 1)
    ring = np.stack([np.zeros_like(th), cy + radius * np.cos(th), cz + radius * np.sin(th)], -1)
    tris = []
    for a in range(n_len):
        for i in range(n_theta):
            j = (i + 1) % n_theta
            p00 = ring[i] + [xs[a], 0, 0]
            p01 = ring[j] + [xs[a], 0, 0]
            p10 = ring[i] + [xs[a + 1], 0, 0]
            p11 = ring[j] + [xs[a + 1], 0, 0]
            tris.append([p00, p11, p10])
            tris.append([p00, p01, p11])
    for x, sgn in ((xs[0], 1), (xs[-1], -1)):
        c = np.array([x, cy, cz])
        for i in range(n_theta):
            j = (i + 1) % n_theta
            a = ring[i] + [x, 0, 0]
            b = ring[j] + [x, 0, 0]
            tris.append([c, a, b] if sgn > 0 else [c, b, a])
    t = np.array(tris, dtype=np.float64)
    # orient inward: normal should point toward the axis / into the cylinder
    nrm = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    cen = t.mean(1)
    inward = np.array(center, dtype=np.float64) - cen
    inward[:, 0] = np.where(np.abs(cen[:, 0] - cx) > length / 2 - 1e-9, cx - cen[:, 0], 0.0)
    side = np.abs(cen[:, 0] - cx) <= length / 2 - 1e-9
    inward[side, 0] = 0.0
    flip = (nrm * inward).sum(-1) < 0
    t[flip] = t[flip][:, [0, 2, 1]]
    return t


def icosphere(center, radius, subdiv=1) -> np.ndarray:
    """Icosphere triangles (20*4^subdiv), normals pointing outward."""
    g = (1 + 5 ** 0.5) / 2
    v = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g), (0, 1, -g),
         (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    v = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]
        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    V = np.array(v) * radius + np.array(center, dtype=np.float64)
    t = V[np.array(f)]
    nrm = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    flip = (nrm * (t.mean(1) - np.array(center))).sum(-1) < 0
    t[flip] = t[flip][:, [0, 2, 1]]
    return t


def _fill_height(radius: float, frac: float) -> float:
    """Height h above the bottom of a horizontal circle whose segment holds frac of
    the area."""
    lo, hi = 0.0, 2 * radius
    for _ in range(80):
        h = 0.5 * (lo + hi)
        d = radius - h
        area = radius * radius * math.acos(d / radius) - d * math.sqrt(max(radius * radius - d * d, 0.0))
        if area / (math.pi * radius * radius) < frac:
            lo = h
        else:
            hi = h
    return 0.5 * (lo + hi)


def _lattice(lo, hi, l0):
    axes = [np.arange(lo[a] + 0.5 * l0, hi[a] - 0.25 * l0, l0) for a in range(3)]
    g = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    return g


def _finish(name, p, pos, tris, models, tparams, drag, seed, l0, zone_lo=None, zone_hi=None) -> Scene:
    rng = np.random.default_rng(seed)
    pos = pos + rng.uniform(-0.01 * l0, 0.01 * l0, size=pos.shape)
    n = pos.shape[0]
    if zone_lo is None:
        # automatic compute zone (MultiGPUHandler.cpp:109-144): bounding box of
        # particles and triangles grown by l0 * max(re)
        allp = np.concatenate([pos, tris.reshape(-1, 3)]) if len(tris) else pos
        off = l0 * max(p.LaplacianInfluenceRadiusCoefficient, p.GradientInfluenceRadiusCoefficient)
        zone_lo = allp.min(0) - off
        zone_hi = allp.max(0) + off
    box = grid_box(zone_lo, zone_hi, p)
    n0g, _ = lattice_constants(p.GradientInfluenceRadiusCoefficient)
    n0l, lam1 = lattice_constants(p.LaplacianInfluenceRadiusCoefficient)
    return Scene(name=name, param=p, box=box, pos=pos.astype(np.float64), vel=np.zeros((n, 3)),
                 press=np.zeros(n), visc=np.full(n, 1e-6), ptype=np.zeros(n, dtype=np.int32),
                 tri_vertices=np.asarray(tris, dtype=np.float64).reshape(-1, 3, 3),
                 tri_model=np.asarray(models, dtype=np.int32), tri_params=tparams, drag=drag,
                 n0_pnd=n0g, n0_lap=n0l, lam=lam1 * l0 * l0)


def dam_break(l0: float = 0.01, dt: float = 1e-4, seed: int = 1, explicit_pressure: bool = False,
              column=(0.2, 0.2, 0.4), tank=(0.8, 0.2, 0.6)) -> Scene:
    p = default_param(l0, dt, explicit_pressure=explicit_pressure)
    # first particle layer at 1.0*l0 from the walls: the wall-weight tables
    # (Z functions) count the missing neighbours of a particle at that distance
    pos = _lattice((0.0, 0.0, 0.0), column, l0)
    h = 0.5 * l0
    tris = box_triangles((-h, -h, -h), (tank[0] - h, tank[1] - h, tank[2] - h))
    models = np.zeros(len(tris), dtype=np.int32)
    tp = [_tri_normal_params(dt=dt)]
    return _finish("dam_break", p, pos, tris, models, tp, [], seed, l0)


def rotating_bucket(l0: float = 0.004, dt: float = 5e-5, seed: int = 2, rpm: float = 30.0, fill: float = 0.35,
                    radius: float = 0.15, length: float = 0.3, n_drag: int = 64, drag_seed: int = 3,
                    explicit_pressure: bool = False, n_theta: int = 64, n_len: int = 31,
                    drag_index: float = 0.5) -> Scene:
    p = default_param(l0, dt, explicit_pressure=explicit_pressure)
    center = (0.0, 0.0, 0.0)
    tris = cylinder_triangles(center, radius, length, n_theta, n_len)
    models = [0] * len(tris)
    h = _fill_height(radius - l0, fill)
    g = _lattice((-length / 2, -radius, -radius), (length / 2, radius, radius), l0)
    r2 = g[:, 1] ** 2 + g[:, 2] ** 2
    keep = (r2 <= (radius - l0) ** 2) & (g[:, 2] <= -radius + l0 + h) & (np.abs(g[:, 0]) <= length / 2 - l0)
    pos = g[keep]
    tparams = [_tri_normal_params(rotating=True, rpm=rpm, dt=dt, center=center, second=(1.0, 0.0, 0.0))]
    drag = []
    if n_drag > 0:
        rng = np.random.default_rng(drag_seed)
        rs = 3.0 * l0
        centers = pos[rng.choice(len(pos), size=n_drag, replace=False)]
        tris_list = [tris]
        for i, c in enumerate(centers):
            s = icosphere(c, rs, subdiv=1)
            tris_list.append(s)
            models += [1] * len(s)
        tris = np.concatenate(tris_list)
        tparams.append(_tri_normal_params(dt=dt, is_drag=True, drag_id=0))
        d = DragParameter()
        d.DragID = 0
        d.DragToken = b"E"
        d.InputVelocityToken1 = b"V"
        d.OutputVelocityToken2 = b"V"
        d.CoefficientofInflueneRegion = 1.0
        d.VelocityIndex = drag_index * dt
        d.VelocityExponential = 1.0
        d.VelocityDragPermiabilityConstant = 1.0
        d.VelocityMagnitueFactor = 1.0
        drag.append(d)
    return _finish("rotating_bucket", p, pos, tris, np.asarray(models), tparams, drag, seed, l0)


def mixer(l0: float = 0.002, dt: float = 5e-5, seed: int = 6, n_drag: int = 512, fill: float = 0.40,
          length: float = 0.3, n_theta: int = 96, n_len: int = 62) -> Scene:
    """Four horizontal buckets side by side along y in one grid."""
    rng = np.random.default_rng(seed)
    radii = rng.uniform(0.10, 0.18, size=4)
    rpms = rng.uniform(20, 45, size=4)
    p = default_param(l0, dt)
    tris_all, models, tparams, pos_all = [], [], [], []
    y = 0.0
    for b in range(4):
        r = float(radii[b])
        y += r
        c = (0.0, y, 0.0)
        t = cylinder_triangles(c, r, length, n_theta, n_len)
        tris_all.append(t)
        models += [b] * len(t)
        tparams.append(_tri_normal_params(rotating=True, rpm=float(int(rpms[b])), dt=dt, center=c,
                                          second=(1.0, y, 0.0)))
        h = _fill_height(r - l0, fill)
        g = _lattice((-length / 2, y - r, -r), (length / 2, y + r, r), l0)
        keep = (((g[:, 1] - y) ** 2 + g[:, 2] ** 2 <= (r - l0) ** 2) & (g[:, 2] <= -r + l0 + h)
                & (np.abs(g[:, 0]) <= length / 2 - l0))
        pos_all.append(g[keep])
        y += r + 8 * l0
    pos = np.concatenate(pos_all)
    drag = []
    if n_drag > 0:
        rs = 3.0 * l0
        centers = pos[rng.choice(len(pos), size=n_drag, replace=False)]
        for c in centers:
            s = icosphere(c, rs, subdiv=0)
            tris_all.append(s)
            models += [4] * len(s)
        tparams.append(_tri_normal_params(dt=dt, is_drag=True, drag_id=0))
        d = DragParameter()
        d.DragToken = b"E"
        d.InputVelocityToken1 = b"V"
        d.OutputVelocityToken2 = b"V"
        d.CoefficientofInflueneRegion = 1.0
        d.VelocityIndex = 0.5 * dt
        d.VelocityExponential = 1.0
        d.VelocityDragPermiabilityConstant = 1.0
        drag.append(d)
    tris = np.concatenate(tris_all)
    return _finish("mixer", p, pos, tris, np.asarray(models), tparams, drag, seed, l0)


def random_block(n_side: int = 12, l0: float = 0.01, seed: int = 0, jitter: float = 0.3,
                 explicit_pressure: bool = True, with_box: bool = True, vel_scale: float = 0.05) -> Scene:
    """Small jittered block of fluid in a box, for kernel parity tests: n_side^3
    particles with jitter*l0 position noise and random velocities."""
    p = default_param(l0, 1e-4, explicit_pressure=explicit_pressure, sonic=10.0)
    p.ArtificialPressure = 1e-3
    p.r_coeff = 1.0
    rng = np.random.default_rng(seed)
    ext = n_side * l0
    pos = _lattice((0, 0, 0), (ext, ext, ext), l0)
    pos = pos + rng.uniform(-jitter * l0, jitter * l0, size=pos.shape)
    tris = box_triangles((-0.5 * l0, -0.5 * l0, -0.5 * l0), (ext + 0.5 * l0, ext + 0.5 * l0, ext + 1.5 * l0)) if with_box \
        else np.zeros((0, 3, 3))
    models = np.zeros(len(tris), dtype=np.int32)
    sc = _finish("random_block", p, pos, tris, models, [_tri_normal_params(dt=p.Dt)], [], seed + 1000, l0)
    sc.vel = rng.normal(0.0, vel_scale, size=sc.pos.shape)
    sc.press = np.abs(rng.normal(0.0, 50.0, size=sc.n))
    return sc
