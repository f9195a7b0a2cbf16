"""The five benchmark workloads of the PIC/DSMC step, built from seeds.

0  plain FP64, CPU-sized: 100 mm cube, 10^3 Kuhn cells (6,000 tets, 1,331
   nodes), 1e4 Ti+ (w = 1e6) from a 20 mm disk, 1 eV, 30 deg cone, Ar 1 Pa HS,
   dt 1e-8 s, 200 steps, Poisson every 10.
1  plain FP64 at scale: 200 mm cube, h = 2 mm (6.0e6 tets, 1.03e6 nodes), 1e7
   Ti+ from the same disk, Thompson energies (U = 4.9 eV, Emax = 50 eV),
   cosine-law directions, Ar 0.5 Pa VHS, dt 5e-9 s, 1,000 steps, Poisson
   every 10, re-sort every 20.
2  workload 1 in the mixed-precision form.
3  jittered 200x200x100 mm box (~1.47e7 tets, ~2.5e6 nodes), plates at
   z = 20 mm (0 V) and 80 mm (-300 V), 5e7 Ti+ from the lower plate, Ar 2 Pa VSS.
4  differentiation: workload 0 at h = 4 mm, six face potentials, 1e6 Ti+.

Units are SI. The gas density is n = P/(R T) N_A as in
util::calculateConcentration (src/Utilities/Utilities.cpp:132-149).
Workloads 1-3 do not name a macro-particle weight, so they use weight 1, the
reference's own semantics (its particles carry their species charge).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import mesh as M
from .sources import make_particles

R_GAS = 8.314  # Constants.hpp:10
N_AV = 6.02214076e23  # Constants.hpp:13
E_CHARGE = 1.602176565e-19  # Constants.hpp e_charge
TI_MASS = 7.95e-26
AR_MASS = 6.6335209e-26  # Constants.hpp Ar_mass
KT_REF = 297.0 * 1.380658e-23  # Constants.hpp:12
EPS0 = 8.8541878128e-12


def gas_concentration(pressure, temperature):
    return (pressure / (R_GAS * temperature)) * N_AV


@dataclass
class Workload:
    name: str
    mesh: M.TetMesh
    params: dict
    pos: np.ndarray
    vel: np.ndarray
    steps: int
    meta: dict = field(default_factory=dict)


def _base_params(**kw):
    p = dict(dt=1e-8, charge=E_CHARGE, mass=TI_MASS, weight=1.0, collision_model=0, precision=0,
             gas_mass=AR_MASS, gas_concentration=0.0, hs_diameter=3.6e-10, vhs_dref=4.17e-10, omega=0.81,
             alpha=1.40, kT_ref=KT_REF, epsilon0=EPS0, min_velocity=10.0, bbox_expansion=1.01, seed=0,
             poisson_every=10, resort_every=20, max_crossings=4096, cg_max_iter=20000, cg_rtol=1e-10, device=0,
             preconditioner=0)
    p.update(kw)
    return p


def _zbc(m: M.TetMesh, v0=0.0, v1=100.0):
    lo = M.box_face_nodes(m, 2, 0)
    hi = M.box_face_nodes(m, 2, 1)
    return m.with_dirichlet(np.concatenate([lo, hi]), np.concatenate([np.full(len(lo), v0), np.full(len(hi), v1)]))


def workload0(n_particles=10_000, cells=10, collisions=True, seed=0, steps=200):
    L = 0.1
    m = _zbc(M.kuhn_box((cells,) * 3, (L,) * 3))
    pos, vel = make_particles(seed, n_particles, TI_MASS, source="disk", centre=(L / 2, L / 2, 0.0), radius=0.02,
                              directions="cone", half_angle=np.deg2rad(30.0), energy="mono", energy_ev=1.0)
    p = _base_params(dt=1e-8, weight=1e6, collision_model=1 if collisions else 0,
                     gas_concentration=gas_concentration(1.0, 300.0), seed=seed, poisson_every=10, resort_every=20)
    return Workload("cube100mm_h10mm_1e4ptcl_HS", m, p, pos, vel, steps,
                    dict(workload=0, cells=cells, n_particles=n_particles))


def workload1(n_particles=10_000_000, cells=100, seed=0, steps=1000, collisions=True):
    L = 0.2
    m = _zbc(M.kuhn_box((cells,) * 3, (L,) * 3))
    pos, vel = make_particles(seed, n_particles, TI_MASS, source="disk", centre=(L / 2, L / 2, 0.0), radius=0.02,
                              directions="cosine", energy="thompson", binding_ev=4.9, emax_ev=50.0)
    p = _base_params(dt=5e-9, weight=1.0, collision_model=2 if collisions else 0,
                     gas_concentration=gas_concentration(0.5, 300.0), seed=seed, poisson_every=10, resort_every=20)
    return Workload(f"cube200mm_h{200 // cells}mm_{n_particles:.0e}ptcl_VHS".replace("+0", ""), m, p, pos, vel,
                    steps, dict(workload=1, cells=cells, n_particles=n_particles))


def workload2(**kw):
    w = workload1(**kw)
    w.params["precision"] = 1
    w.meta["workload"] = 2
    w.name += "_mixed"
    return w


def workload3(n_particles=50_000_000, cells=(170, 170, 85), seed=0, steps=2000, jitter_frac=0.2):
    Lx, Ly, Lz = 0.2, 0.2, 0.1
    m = M.kuhn_box(cells, (Lx, Ly, Lz))
    xl, yl = (0.06, 0.14), (0.06, 0.14)
    low = M.add_plate(m, 0.02, xl, yl, tag=7)
    high = M.add_plate(m, 0.08, xl, yl, tag=8)
    M.jitter(m, jitter_frac, seed=seed + 11, frozen=np.concatenate([low, high]))
    m.with_dirichlet(np.concatenate([low, high]), np.concatenate([np.zeros(len(low)), np.full(len(high), -300.0)]))
    pos, vel = make_particles(seed, n_particles, TI_MASS, source="plate", xlim=xl, ylim=yl, z=0.02,
                              directions="cosine", energy="thompson", binding_ev=4.9, emax_ev=50.0)
    p = _base_params(dt=5e-9, weight=1.0, collision_model=3, gas_concentration=gas_concentration(2.0, 300.0),
                     seed=seed, poisson_every=10, resort_every=20, precision=1)
    return Workload("box200x200x100_jitter_plates_VSS", m, p, pos, vel, steps,
                    dict(workload=3, cells=cells, n_particles=n_particles))


def workload4(n_particles=1_000_000, cells=25, seed=1, steps=300, potentials=None, half_angle_deg=30.0):
    L = 0.1
    m = M.kuhn_box((cells,) * 3, (L,) * 3)
    rng = np.random.default_rng(seed)
    V = rng.uniform(-100.0, 100.0, 6) if potentials is None else np.asarray(potentials, float)
    nodes, vals = [], []
    for f, (ax, side) in enumerate(M.BOX_FACES):
        nd = M.box_face_nodes(m, ax, side)
        nodes.append(nd)
        vals.append(np.full(len(nd), V[f]))
    m.with_dirichlet(np.concatenate(nodes), np.concatenate(vals))  # later faces win on shared edges
    pos, vel = make_particles(seed, n_particles, TI_MASS, source="disk", centre=(L / 2, L / 2, 0.0), radius=0.02,
                              directions="cone", half_angle=np.deg2rad(half_angle_deg), energy="mono", energy_ev=1.0)
    p = _base_params(dt=1e-8, weight=1e6, collision_model=0, seed=seed, poisson_every=10, resort_every=20)
    return Workload("cube100mm_h4mm_1e6ptcl_grad", m, p, pos, vel, steps,
                    dict(workload=4, potentials=V.tolist(), half_angle_deg=half_angle_deg))


WORKLOADS = {0: workload0, 1: workload1, 2: workload2, 3: workload3, 4: workload4}
