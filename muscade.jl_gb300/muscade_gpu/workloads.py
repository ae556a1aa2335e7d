"""Synthetic models of the benchmark configurations (seeded, reproducible).

* cantilever(): 10 m beam of 20 EulerBeam3D along x, clamped with six Hold at
  node 1, tip DofLoad in t3 ramping to 1e3 N, SweepX{0} over 10 load steps.
* lattice(nx, ny, nz): 3D frame of EulerBeam3D on all edges of a 1 m grid,
  section properties lognormal (σ=0.1) around the cantilever's, all six dofs
  held on the z=0 layer, Gaussian (σ=100 N) DofLoads on every free
  translation ramped by t.  60×60×20 gives 210,000 beams.
* risers(nriser, nel): independent vertical risers of 1000 m, pinned at the
  bottom (Hold t1,t2,t3,r1) and driven at the top by DofConstraints
  t1 = A sin(2πt/T)·ρ(t), t2 = 0, t3 = 0.1 m·ρ(t) (pretension), A~U(1,5),
  T~U(8,15), with ρ a cosine ramp from 0 to 1 over the first 5 s.

Random streams use numpy PCG64 with seed 2026 + configuration index.
"""
from __future__ import annotations

import math

import numpy as np

from .elements import (BeamCrossSection, DofConstraint, DofLoad, EulerBeam3D, Hold, QuadraticCost, SingleAcost,
                       SingleDofCost)
from .model import Model

EA0, EI0, GJ0, MU0, IOTA0 = 1e8, 1e4, 1e4, 10.0, 1.0


def cantilever(nel=20, length=10.0, load=1e3):
    m = Model("cantilever")
    xs = np.linspace(0.0, length, nel + 1)
    nodes = m.addnode(np.stack([xs, np.zeros_like(xs), np.zeros_like(xs)], axis=1))
    mat = BeamCrossSection(EA=EA0, EI2=EI0, EI3=EI0, GJ=GJ0, mu=MU0, iota1=IOTA0)
    m.addelement(EulerBeam3D, np.stack([nodes[:-1], nodes[1:]], axis=1), mat=mat, orient2=(0.0, 1.0, 0.0))
    for f in ("t1", "t2", "t3", "r1", "r2", "r3"):
        m.addelement(Hold, [nodes[0]], field=f)

    def tipload(t):
        return load * t

    m.addelement(DofLoad, [nodes[-1]], field="t3", value=tipload)
    return m, np.round(np.arange(1, 11) * 0.1, 12)


def bend45(nel=8, radius=100.0):
    """The 45° cantilever bend of examples/StaticBeamAnalysis.jl:10-36: a
    circular arc of radius 100 m in the x-z plane, 8 EulerBeam3D (EA 1e9 N,
    EI₂ = EI₃ = 833.33e3 N·m², GJ 705e3 N·m²), clamped at the first node, an
    out-of-plane tip load along y ramped to 300, 450 and 600 N at t = 1, 2, 3.
    Returns the model, the load times (0, 1, 2, 3) and the tip node."""
    m = Model("bend45")
    a = 1.5 * math.pi + np.arange(nel + 1) / nel * (math.pi / 4)
    xyz = np.stack([radius * np.cos(a), np.zeros(nel + 1), radius + radius * np.sin(a)], axis=1)
    nodes = m.addnode(xyz)
    mat = BeamCrossSection(EA=1e9, EI2=833.33e3, EI3=833.33e3, GJ=705e3, mu=1.0, iota1=1.0)
    m.addelement(EulerBeam3D, np.stack([nodes[:-1], nodes[1:]], axis=1), mat=mat, orient2=(0.0, 1.0, 0.0))
    for f in ("t1", "t2", "t3", "r1", "r2", "r3"):
        m.addelement(Hold, [nodes[0]], field=f)

    def load(t):
        return t * 300.0 if t <= 1.0 else (300.0 + (t - 1.0) * 150.0 if t <= 2.0 else 450.0 + (t - 2.0) * 150.0)

    m.addelement(DofLoad, [nodes[-1]], field="t2", value=load)
    return m, [0.0, 1.0, 2.0, 3.0], int(nodes[-1])


def lattice(nx=60, ny=60, nz=20, seed=2027, sigma=0.1, load_std=100.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    m = Model("lattice")
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    nid = np.zeros((nx, ny, nz), dtype=np.int64)
    coords = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], axis=1).astype(np.float64)
    ids = m.addnode(coords)
    nid[I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")] = ids
    edges = []
    orients = []
    # x-, y- and z-edges; orient2 chosen so that no as-meshed frame is a half turn
    e = np.stack([nid[:-1, :, :].ravel(order="F"), nid[1:, :, :].ravel(order="F")], axis=1)
    edges.append(e)
    orients.append((0.0, 1.0, 0.0))
    e = np.stack([nid[:, :-1, :].ravel(order="F"), nid[:, 1:, :].ravel(order="F")], axis=1)
    edges.append(e)
    orients.append((0.0, 0.0, 1.0))
    e = np.stack([nid[:, :, :-1].ravel(order="F"), nid[:, :, 1:].ravel(order="F")], axis=1)
    edges.append(e)
    orients.append((1.0, 0.0, 0.0))
    nbeam = sum(len(e) for e in edges)
    ln = lambda: np.exp(rng.normal(0.0, sigma, nbeam))  # noqa: E731
    EA, EI2, EI3, GJ = EA0 * ln(), EI0 * ln(), EI0 * ln(), GJ0 * ln()
    p = 0
    for e, o in zip(edges, orients):
        sl = slice(p, p + len(e))
        mat = BeamCrossSection(EA=EA[sl], EI2=EI2[sl], EI3=EI3[sl], GJ=GJ[sl], mu=MU0, iota1=IOTA0)
        m.addelement(EulerBeam3D, e, mat=mat, orient2=o)
        p += len(e)
    base = nid[:, :, 0].ravel(order="F")
    for f in ("t1", "t2", "t3", "r1", "r2", "r3"):
        m.addelement(Hold, base[:, None], field=f)
    free = nid[:, :, 1:].ravel(order="F")
    for f in ("t1", "t2", "t3"):
        F = rng.normal(0.0, load_std, len(free))

        def ramp(t, F=F):
            return F * t

        m.addelement(DofLoad, free[:, None], field=f, value=ramp)
    return m, np.round(np.arange(1, 6) * 0.2, 12)


def risers(nriser=200, nel=250, length=1000.0, seed=2028, EA=5e9, EI=1e6, GJ=1e6, mu=300.0, iota1=10.0,
           subset=None):
    """`nriser` seeded risers; `subset` = (lo, hi) builds only risers lo..hi-1 of
    them (the amplitudes and periods are drawn for all, so a subset's risers are
    those of the whole set)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.uniform(1.0, 5.0, nriser)
    T = rng.uniform(8.0, 15.0, nriser)
    lo, hi = subset if subset is not None else (0, nriser)
    A, T = A[lo:hi], T[lo:hi]
    m = Model("risers")
    mat = BeamCrossSection(EA=EA, EI2=EI, EI3=EI, GJ=GJ, mu=mu, iota1=iota1)
    zs = np.linspace(0.0, length, nel + 1)
    bottoms, tops = [], []
    for r in range(lo, hi):
        x0 = 50.0 * (r % 20)
        y0 = 50.0 * (r // 20)
        nodes = m.addnode(np.stack([np.full_like(zs, x0), np.full_like(zs, y0), zs], axis=1))
        m.addelement(EulerBeam3D, np.stack([nodes[:-1], nodes[1:]], axis=1), mat=mat, orient2=(1.0, 0.0, 0.0))
        bottoms.append(nodes[0])
        tops.append(nodes[-1])
    bottoms = np.asarray(bottoms)[:, None]
    tops = np.asarray(tops)[:, None]
    for f in ("t1", "t2", "t3", "r1"):
        m.addelement(Hold, bottoms, field=f)

    def ramp(t):  # smooth start of the prescribed top motion over the first 5 s
        return 0.5 * (1.0 - math.cos(math.pi * min(t, 5.0) / 5.0))

    def surge(t):
        return A * np.sin(2 * math.pi * t / T) * ramp(t)

    def zero(t):
        return 0.0

    def lift(t):
        return 0.1 * ramp(t)

    m.addelement(DofConstraint, tops, xinod=(1,), xfield=("t1",), lfield="λtop1", coeffs=[1.0], offset=surge, name="surge")
    m.addelement(DofConstraint, tops, xinod=(1,), xfield=("t2",), lfield="λtop2", coeffs=[1.0], offset=zero, name="sway")
    m.addelement(DofConstraint, tops, xinod=(1,), xfield=("t3",), lfield="λtop3", coeffs=[1.0], offset=lift, name="lift")
    return m, 0.05 * np.arange(1, 2001)


# ---------------------------------------------------------------- batched models
def batched_params(nmodel=4096, nel_range=(10, 400), seed=2030, sigma=0.15):
    """Parameters of independent models for one batched solve: half
    cantilevers with the section of the 10 m one above but 2 m long (tip
    DofLoad in t3; at 5 m and 10 m plain Newton from the straight beam
    diverges in the first load step for the finer meshes and larger loads --
    the first linear step stretches the short elements -- in the oracle as on
    the device), half portal frames
    (two 5 m columns and a 10 m beam, both bases held in all six dofs,
    mid-span DofLoad in -t3).  Element counts U{nel_range}; EA, EI2, EI3, GJ
    the cantilever's times lognormal(0, sigma) per model; load Gumbel with mode
    1e3 N and scale 200 N, ramped by t."""
    rng = np.random.Generator(np.random.PCG64(seed))
    portal = rng.random(nmodel) < 0.5
    nel = rng.integers(nel_range[0], nel_range[1] + 1, nmodel)
    ln = np.exp(rng.normal(0.0, sigma, (nmodel, 4)))
    load = rng.gumbel(1e3, 200.0, nmodel)
    return [dict(kind="portal" if portal[i] else "cantilever", nel=int(nel[i]), EA=EA0 * ln[i, 0], EI2=EI0 * ln[i, 1],
                 EI3=EI0 * ln[i, 2], GJ=GJ0 * ln[i, 3], load=float(load[i])) for i in range(nmodel)]


def _model_geometry(p):
    """Node coordinates (local), beam connectivity (local, 1-based), held nodes, loaded node, load sign."""
    nel = p["nel"]
    if p["kind"] == "cantilever":
        xs = np.linspace(0.0, 2.0, nel + 1)
        xyz = np.stack([xs, np.zeros_like(xs), np.zeros_like(xs)], axis=1)
        conn = np.stack([np.arange(1, nel + 1), np.arange(2, nel + 2)], axis=1)
        return xyz, conn, [1], nel + 1, 1.0
    H, B = 5.0, 10.0
    ncol = max(1, nel // 4)
    nbeam = nel - 2 * ncol
    if nbeam % 2:  # even beam element count: a node at mid-span
        ncol, nbeam = ncol + 1, nbeam - 1
    if nbeam < 2:
        ncol, nbeam = (nel - 2) // 2, 2 + (nel - 2) % 2
    left = np.stack([np.zeros(ncol + 1), np.zeros(ncol + 1), np.linspace(0.0, H, ncol + 1)], axis=1)
    top = np.stack([np.linspace(0.0, B, nbeam + 1)[1:], np.zeros(nbeam), np.full(nbeam, H)], axis=1)
    right = np.stack([np.full(ncol, B), np.zeros(ncol), np.linspace(H, 0.0, ncol + 1)[1:]], axis=1)
    xyz = np.concatenate([left, top, right])
    nn = len(xyz)
    conn = np.stack([np.arange(1, nn), np.arange(2, nn + 1)], axis=1)
    mid = ncol + 1 + nbeam // 2
    return xyz, conn, [1, nn], mid, -1.0


def build_batched(params, spacing=30.0):
    """One Model holding the given independent models (disjoint node sets, side
    by side in y).  Returns (model, node_offset per model, load times)."""
    m = Model("batched")
    geo = [_model_geometry(p) for p in params]
    xyz, conn, held, loaded, sign, offs = [], [], [], [], [], []
    mats = {k: [] for k in ("EA", "EI2", "EI3", "GJ")}
    off = 0
    for i, (p, (x, c, h, ld, sg)) in enumerate(zip(params, geo)):
        x = x.copy()
        x[:, 1] += spacing * i
        xyz.append(x)
        conn.append(c + off)
        held += [hh + off for hh in h]
        loaded.append(ld + off)
        sign.append(sg * p["load"])
        for k in mats:
            mats[k].append(np.full(len(c), p[k]))
        offs.append(off)
        off += len(x)
    m.addnode(np.concatenate(xyz))
    mat = BeamCrossSection(EA=np.concatenate(mats["EA"]), EI2=np.concatenate(mats["EI2"]),
                           EI3=np.concatenate(mats["EI3"]), GJ=np.concatenate(mats["GJ"]), mu=MU0, iota1=IOTA0)
    m.addelement(EulerBeam3D, np.concatenate(conn), mat=mat, orient2=(0.0, 1.0, 0.0))
    held = np.asarray(held)[:, None]
    for f in ("t1", "t2", "t3", "r1", "r2", "r3"):
        m.addelement(Hold, held, field=f)
    F = np.asarray(sign)

    def ramp(t, F=F):
        return F * t

    m.addelement(DofLoad, np.asarray(loaded)[:, None], field="t3", value=ramp)
    return m, np.asarray(offs), np.round(np.arange(1, 9) * 0.125, 12)


def node_dofs(model, nodes):
    """X-dof indices (0-based) of every X dof type at the given nodes, in dof-type order; -1 where absent."""
    nodes = np.asarray(nodes, dtype=np.int64)
    xt = [i for i, d in enumerate(model.doftyp) if d.cls == "X"]
    return model._ndmap[nodes[:, None] - 1, np.asarray(xt)[None, :]] - 1


# ---------------------------------------------------------------- identification
def adjoint_beam(nel=5000, nstep=500, dt=0.01, seed=2029, ele_len=0.1, EA=1e10, EI=1e8, GJ=1e8, mu=1e3, iota1=10.0,
                 load_std=1e3, corr_x=10.0, corr_t=0.2, nfeat=64, sigma_A=0.2, sensor_frac=0.05, measurements=None,
                 a_weight=0.0):
    """Simply supported beam for load and stiffness identification: nel
    EulerBeam3D{adof} of ele_len along x, one EI-scale A-dof per element (on its
    own parameter node), Hold t1, t2, t3 at both ends and r1 at the first node,
    a DofLoad in t2 at every interior node whose values are a Gaussian process
    in space (correlation length corr_x) and time (corr_t), drawn with nfeat
    random Fourier features.  Returns a dict with the model, the time grid,
    the load table, the true A (lognormal, sigma_A) and the sensor dofs
    (a random sensor_frac of the free translational dofs, 1-based).

    With measurements = (y, sd) (y[nstep][nsensor], as synthetic_measurements
    returns), the model also carries the identification cost as elements: a
    SingleDofCost per sensor with QuadraticCost(1/sd², yₛ(t)) and, when
    a_weight > 0, a SingleAcost QuadraticCost(a_weight, 1) on every A-dof."""
    rng = np.random.Generator(np.random.PCG64(seed))
    m = Model("identification")
    xs = np.arange(nel + 1) * ele_len
    nodes = m.addnode(np.stack([xs, np.zeros_like(xs), np.zeros_like(xs)], axis=1))
    pnodes = m.addnode(np.stack([(xs[:-1] + xs[1:]) / 2, np.full(nel, 1.0), np.zeros(nel)], axis=1))
    mat = BeamCrossSection(EA=EA, EI2=EI, EI3=EI, GJ=GJ, mu=mu, iota1=iota1)
    m.addelement(EulerBeam3D, np.stack([nodes[:-1], nodes[1:], pnodes], axis=1), mat=mat, orient2=(0.0, 1.0, 0.0),
                 adof=True)
    for f in ("t1", "t2", "t3"):
        m.addelement(Hold, np.array([[nodes[0]], [nodes[-1]]]), field=f)
    m.addelement(Hold, [nodes[0]], field="r1")
    times = np.round(np.arange(1, nstep + 1) * dt, 12)
    inner = nodes[1:-1]
    wx = rng.normal(0.0, 1.0 / corr_x, nfeat)
    wt = rng.normal(0.0, 1.0 / corr_t, nfeat)
    ph = rng.uniform(0.0, 2 * math.pi, nfeat)
    amp = load_std * math.sqrt(2.0 / nfeat)
    xi = xs[1:-1]
    table = np.zeros((nstep, len(inner)))
    for k in range(nfeat):
        table += amp * np.cos(wx[k] * xi[None, :] + wt[k] * times[:, None] + ph[k])

    def load(t, table=table, dt=dt):
        k = int(round(t / dt)) - 1
        return table[k] if 0 <= k < len(table) else np.zeros(table.shape[1])

    m.addelement(DofLoad, inner[:, None], field="t2", value=load)
    A_true = np.exp(rng.normal(0.0, sigma_A, nel))
    cand = node_dofs(m, nodes)[:, :3]  # t1, t2, t3 of the beam nodes
    held = {(int(nodes[0]), 0), (int(nodes[0]), 1), (int(nodes[0]), 2), (int(nodes[-1]), 0), (int(nodes[-1]), 1),
            (int(nodes[-1]), 2)}
    free = [cand[i, j] for i in range(len(nodes)) for j in range(3) if (int(nodes[i]), j) not in held]
    nsens = max(1, int(round(sensor_frac * len(free))))
    sensors = np.sort(rng.choice(np.asarray(free), nsens, replace=False)) + 1
    if measurements is not None:
        y, sd = measurements
        identification_costs(m, sensors, y, sd, times, pnodes if a_weight > 0 else None, a_weight)
    return dict(model=m, times=times, loads=table, A_true=A_true, sensors=sensors, nodes=nodes, pnodes=pnodes,
                seed=seed)


class _Record:
    """y(t) of one sensor from its record on the time grid (zero off the grid)."""

    def __init__(self, times, values):
        self.index = {round(float(t), 12): k for k, t in enumerate(times)}
        self.values = np.asarray(values, dtype=np.float64)

    def __call__(self, t):
        k = self.index.get(round(float(t), 12))
        return 0.0 if k is None else float(self.values[k])


def identification_costs(model, sensors, y, sd, times, anodes=None, a_weight=0.0):
    """Adds a SingleDofCost QuadraticCost(1/sd², yₛ(t)) on each sensor dof
    (1-based X-dofs, records y[nstep][nsensor]) and, with anodes, a SingleAcost
    QuadraticCost(a_weight, 1) on the EIscale A-dof of each of those nodes."""
    for s, dof in enumerate(np.asarray(sensors)):
        node = int(model.dof_node["X"][dof - 1])
        field = model.doftyp[model.dof_typ["X"][dof - 1]].field
        model.addelement(SingleDofCost, [node], cls="X", field=field,
                         cost=QuadraticCost(1.0 / sd**2, _Record(times, y[:, s])))
    if anodes is not None:
        model.addelement(SingleAcost, np.asarray(anodes)[:, None], field="EIscale", cost=QuadraticCost(a_weight, 1.0))


def synthetic_measurements(states, sensors, noise=0.01, seed=2031):
    """Sensor records from states[nstep][nder][nX] plus Gaussian noise at
    `noise` times the RMS of the noise-free records."""
    rng = np.random.Generator(np.random.PCG64(seed))
    y = states[:, 0, np.asarray(sensors) - 1]
    rms = math.sqrt(float(np.mean(y * y))) or 1.0
    return y + rng.normal(0.0, noise * rms, y.shape), noise * rms
