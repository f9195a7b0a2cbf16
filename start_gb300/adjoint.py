"""Gradient of the smoothed landing objective (the 100 mm electrode cube).

Parameters: six electrode potentials, one per face of the 100 mm cube, and
the half-angle of the source cone. The forward pass solves the field of the
electrodes (one CG solve), launches the particles from a 20 mm disk on
z = 0 with directions reparameterised by fixed uniforms,
    cos(theta) = 1 - u1 (1 - cos(alpha)),  psi = 2 pi u2,
steps them (collision events and random numbers fixed), and evaluates
    J = mean over landed particles of exp(-|r_land - r_target|^2 / (2 sigma^2)),
with r_target the centre of the z = 100 mm face. The backward pass is the
library's adjoint: the particle adjoint with checkpoint-window recompute, one
adjoint CG on the same stiffness matrix, the transpose of the Dirichlet
lifting; dJ/dalpha follows from dJ/d(initial state) by the chain rule.

The map differentiated is the step with the collision events, the random
numbers and the cell whose E pushes a particle at each step held fixed (the
pathwise derivative). The live step also moves when a push position crosses a
cell face, where the per-cell constant field jumps; central differences of the
live map include those jumps. With field_gradient the backward pass adds the
push's dependence on the position through a continuous field recovered from
the per-tet E, which accounts for most of them.
"""
from __future__ import annotations

import numpy as np

from . import mesh as M
from .engine import StartPIC
from .sources import EV_J, DISPLACEMENT, disk_points
from .workloads import TI_MASS, _base_params, gas_concentration


class LandingSetup:
    """Geometry, electrodes, parameters and the frozen source uniforms of the
    landing problem; no device state (the oracle tests reuse it).

    faces: the box faces (indices into mesh.BOX_FACES) that carry an
    electrode, one potential each; the other faces are Neumann. With only the
    two z faces the field is uniform: P1 reproduces the linear potential
    exactly.

    field_gradient: the backward pass also carries the push's dependence on
    the particle's position through the gradient of a continuous field
    recovered from the per-tet E (spg_grad_field_gradient). Off, the gradient
    is the exact derivative of the map with the pushing cells held fixed; on,
    it follows central differences of the live step much more closely where
    the field varies from cell to cell."""

    def __init__(self, n_particles=1_000_000, cells=25, steps=300, seed=1, sigma=0.01, checkpoint_every=32,
                 collisions=True, energy_ev=1.0, gas_scale=1.0, cg_rtol=1e-12, preconditioner=0, precision=0,
                 faces=(0, 1, 2, 3, 4, 5), field_gradient=False):
        L = 0.1
        self.mesh = M.kuhn_box((cells,) * 3, (L,) * 3)
        self.faces = tuple(faces)
        self.field_gradient = field_gradient
        owner = np.full(self.mesh.n_nodes, -1)
        for f, (ax, side) in enumerate(M.BOX_FACES):
            if f in self.faces:
                owner[M.box_face_nodes(self.mesh, ax, side)] = self.faces.index(f)  # later faces win on edges
        self.owner = owner
        dn = np.nonzero(owner >= 0)[0].astype(np.int32)
        self.mesh.with_dirichlet(dn, np.zeros(len(dn)))
        self.steps, self.sigma, self.every = steps, sigma, checkpoint_every
        self.target = np.array([L / 2, L / 2, L])
        self.params = _base_params(dt=1e-8, weight=1e6, seed=seed, collision_model=1 if collisions else 0,
                                   gas_concentration=gas_concentration(1.0, 300.0) * gas_scale, cg_rtol=cg_rtol,
                                   resort_every=0, preconditioner=preconditioner, precision=precision)
        rng = np.random.default_rng(seed)
        self.p_disk = disk_points(rng, n_particles, (L / 2, L / 2, 0.0), 0.02)
        self.u1 = rng.random(n_particles)
        self.psi = 2.0 * np.pi * rng.random(n_particles)
        self.speed = np.sqrt(2.0 * energy_ev * EV_J / TI_MASS)

    # -- source and its derivative in alpha
    def initial_state(self, alpha):
        ct = 1.0 - self.u1 * (1.0 - np.cos(alpha))
        st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
        d = np.stack([-st * np.sin(self.psi), st * np.cos(self.psi), ct], axis=1)
        dct = -self.u1 * np.sin(alpha)
        dst = np.where(st > 0, -ct * dct / np.where(st > 0, st, 1.0), 0.0)
        dd = np.stack([-dst * np.sin(self.psi), dst * np.cos(self.psi), dct], axis=1)
        # ParticleDisplacer rule: shift by d / max|d_k| * 0.05 mm
        k = np.argmax(np.abs(d), axis=1)
        rows = np.arange(len(d))
        m = np.abs(d[rows, k])
        dm = np.sign(d[rows, k]) * dd[rows, k]
        x0 = self.p_disk + d / m[:, None] * DISPLACEMENT
        dx0 = (dd / m[:, None] - d * (dm / (m * m))[:, None]) * DISPLACEMENT
        return x0, d * self.speed, dx0, dd * self.speed

    def dirichlet_values(self, V):
        g = np.zeros(self.mesh.n_nodes)
        on = self.owner >= 0
        g[on] = np.asarray(V, float)[self.owner[on]]
        return g

    def face_sums(self, dJ_dg):
        return np.array([dJ_dg[self.owner == f].sum() for f in range(len(self.faces))])


class LandingProblem(LandingSetup):
    """The landing problem on the GPU library."""

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        self.engine = StartPIC(self.mesh, self.params)
        self.engine.grad_field_gradient(self.field_gradient)
        self._last = None

    def forward(self, V, alpha):
        e = self.engine
        e.set_dirichlet(self.dirichlet_values(V))
        x0, v0, dx0, dv0 = self.initial_state(alpha)
        e.set_particles(x0, v0)
        e.solve(np.zeros(self.mesh.n_nodes))  # electrode field, no space charge
        J, n_landed = e.grad_forward(self.steps, self.target, self.sigma, self.every)
        self._last = (dx0, dv0, n_landed)
        return J

    def backward(self):
        dx0, dv0, _ = self._last
        dJ_dg, dJ_dx, dJ_dv, iters = self.engine.grad_backward(particles=True)
        dV = self.face_sums(dJ_dg)
        dalpha = float(np.sum(dJ_dx * dx0) + np.sum(dJ_dv * dv0))
        return dV, dalpha, iters

    def close(self):
        self.engine.close()


def landing_objective():
    """torch.autograd.Function over a LandingProblem: params = [V_1..V_k, alpha],
    one potential per electrode face.

    Its gradient is the pathwise derivative: collision events, random numbers
    and the cell whose E pushes each particle at each step are held fixed.
    Where the field is uniform (electrodes on two opposite faces only) it is
    also the derivative of the live step; with a field that varies from cell to
    cell, central differences of the live step differ from it by the jumps of
    the per-cell field (bench.py's grad object records that gap)."""
    import torch

    class LandingObjective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, problem):
            p = params.detach().cpu().double().numpy()
            nf = len(problem.faces)
            J = problem.forward(p[:nf], p[nf])
            ctx.problem = problem
            return torch.tensor(J, dtype=params.dtype, device=params.device)

        @staticmethod
        def backward(ctx, grad_out):
            dV, dalpha, _ = ctx.problem.backward()
            g = torch.tensor(np.concatenate([dV, [dalpha]]), dtype=grad_out.dtype, device=grad_out.device)
            return g * grad_out, None

    return LandingObjective
