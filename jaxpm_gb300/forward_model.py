"""The differentiable forward model: white noise and cosmological
parameters -> Gaussian initial field -> LPT particles -> FastPM steps, with
gradients with respect to the noise field and to ``theta = [Omega_c,
sigma8]``.

This is what ``jax.grad`` computes through ``jaxpm.pm.linear_field``
(``jaxpm/pm.py:129-144``), ``jaxpm.pm.lpt`` (``:61-126``) and the FastPM
integrator (``jaxpm/ode.py:13-82``).  The field and particle operators use
the library's hand-written adjoints (colouring, 2LPT source, forces, the
fused step); the cosmology enters only through host-side scalars (the LPT
growth factors and rates, the per-step kick/drift coefficients) and the
linear power table, and their derivatives with respect to ``theta`` are
taken on the host:

- the scalars: central differences in float64 of the host functions
  (``_HostScalars``; the growth tables come from a fixed-step RK4
  integration, smooth in ``theta``);
- the power table: ``sigma8`` scales the field exactly (``P`` is
  proportional to ``sigma8^2``), so its cotangent is ``<g, ic> / sigma8``;
  ``Omega_c`` changes the transfer function, and its cotangent is
  ``<g, d ic / d Omega_c>`` with the derivative field from two colourings
  at ``Omega_c +- h``.

Parameters are a float64 CPU tensor ``theta`` of two entries; fields and
particles are float32 CUDA tensors.
"""
import dataclasses

import numpy as np
import torch

from . import cosmology as cm
from . import growth as gr
from . import painting, pm, simulate
from .distributed import uniform_particles
from .ode import fpm_coefficients


def cosmology_of(theta, base=None):
    """``base`` (default Planck15) with ``Omega_c, sigma8 = theta``."""
    base = cm.Planck15() if base is None else base
    th = [float(v) for v in np.asarray(theta, dtype=np.float64).reshape(-1)]
    return dataclasses.replace(base, Omega_c=th[0], sigma8=th[1])


class _HostScalars(torch.autograd.Function):
    """``theta -> fn(theta)`` evaluated on the host in float64; the backward
    is the transposed Jacobian from central differences (relative step
    ``rel_step``)."""

    @staticmethod
    def forward(ctx, theta, fn, rel_step):
        th = theta.detach().cpu().double().numpy().copy()
        ctx.fn, ctx.th, ctx.h = fn, th, rel_step
        return torch.tensor(np.asarray(fn(th), dtype=np.float64))

    @staticmethod
    def backward(ctx, g):
        g = g.detach().cpu().double().numpy()
        grad = np.zeros_like(ctx.th)
        for j in range(ctx.th.size):
            h = ctx.h * max(1.0, abs(ctx.th[j]))
            tp, tm = ctx.th.copy(), ctx.th.copy()
            tp[j] += h
            tm[j] -= h
            grad[j] = float(g @ ((np.asarray(ctx.fn(tp)) - np.asarray(ctx.fn(tm))) / (2 * h)))
        return torch.tensor(grad, dtype=torch.float64), None, None


class _LinearField(torch.autograd.Function):
    """``(noise, theta) -> ic``: the noise coloured by the linear power of
    ``cosmology_of(theta)`` (``pm.linear_field``)."""

    @staticmethod
    def forward(ctx, noise, theta, box, base, omega_step):
        th = theta.detach().cpu().double().numpy().copy()
        noise = noise.to(torch.float32).contiguous()
        table = pm.power_table(*pm.pk_table(cosmology_of(th, base)), noise.device)
        ic = pm.colour(noise, table, box)
        ctx.save_for_backward(noise, ic)
        ctx.table, ctx.th, ctx.box, ctx.base, ctx.h = table, th, box, base, omega_step
        return ic

    @staticmethod
    def backward(ctx, g):
        noise, ic = ctx.saved_tensors
        g = g.to(torch.float32).contiguous()
        g_noise = pm.colour(g, ctx.table, ctx.box) if ctx.needs_input_grad[0] else None
        g_theta = None
        if ctx.needs_input_grad[1]:
            th, h = ctx.th, ctx.h
            fields = []
            for sgn in (1.0, -1.0):
                t = th.copy()
                t[0] += sgn * h
                tab = pm.power_table(*pm.pk_table(cosmology_of(t, ctx.base)), noise.device)
                fields.append(pm.colour(noise, tab, ctx.box))
            d_omega = (fields[0].double() - fields[1].double()) / (2 * h)
            gd = g.double()
            g_theta = torch.tensor([float((gd * d_omega).sum()),
                                    float((gd * ic.double()).sum()) / th[1]],
                                   dtype=torch.float64)
        return g_noise, g_theta, None, None, None


def _scalars(theta, base, a0, a1, n_steps, order):
    """[D1, c1, D2, c2, kick_0..kick_{n-1}, drift_0..drift_{n-1}] with
    dx = D1 F1 + D2 F2 and p = c1 F1 + c2 F2 (``jaxpm/pm.py:78-124``)."""
    c = cosmology_of(theta, base)
    a = float(a0)
    E = float(gr.E(c, a))
    D1 = float(gr.growth_factor(c, a))
    f1 = float(gr.growth_rate(c, a))
    out = [D1, a**2 * f1 * E * D1, 0.0, 0.0]
    if order == 2:
        D2 = 3.0 / 7.0 * float(gr.growth_factor_second(c, a))
        f2 = float(gr.growth_rate_second(c, a))
        out[2:] = [D2, a**2 * f2 * E * D2]
    kick, drift = fpm_coefficients(c, a0, a1, n_steps)
    return np.concatenate([out, kick, drift])


def lpt_nbody(noise, theta, mesh_shape, box_size, a0=0.1, a1=1.0, n_steps=32, order=2,
              checkpoint_every=4, base=None, paint_mode="atomic", r_split=0.0,
              omega_step=1e-3, scalar_step=1e-5, engine="sorted"):
    """Final ``(pos, vel)`` of the forward model: ``linear_field`` of
    ``noise`` at ``cosmology_of(theta)``, LPT of order ``order`` at ``a0``
    on the mesh lattice, then ``n_steps`` FastPM steps to ``a1`` with a
    checkpoint every ``checkpoint_every`` steps.  Differentiable with
    respect to ``noise`` and ``theta``.  ``engine`` picks the steps'
    implementation (``simulate.nbody``): ``"sorted"`` (the tile-sorted
    engine, segment by segment; it records a segment's force meshes for the
    backward pass, 3.8 GB per step at 512^3) or ``"lattice"`` (step by step,
    one position array per step kept)."""
    mesh_shape = tuple(int(s) for s in mesh_shape)
    box = tuple(float(b) for b in box_size)
    theta = torch.as_tensor(theta, dtype=torch.float64)
    ic = _LinearField.apply(noise, theta, box, base, omega_step)
    # the LPT and step scalars depend on Omega_c only (sigma8 enters P(k) alone)
    s8 = float(theta[1].detach())
    sc = _HostScalars.apply(
        theta[:1], lambda om: _scalars([om[0], s8], base, a0, a1, n_steps, order), scalar_step)
    lat = uniform_particles(mesh_shape, device=noise.device).reshape(-1, 3)
    F1 = pm.pm_forces(lat, delta=ic, paint_mode=paint_mode)
    dx = sc[0] * F1
    p = sc[1] * F1
    if order == 2:
        F2 = pm.pm_forces(lat, delta=pm._Source2LPT.apply(ic), paint_mode=paint_mode)
        dx = dx + sc[2] * F2
        p = p + sc[3] * F2
    x = (lat + dx).to(torch.float32).contiguous()
    v = p.to(torch.float32).contiguous()
    kick, drift = sc[4:4 + n_steps], sc[4 + n_steps:]
    return simulate.nbody(x, v, None, mesh_shape, a0, a1, n_steps, paint_mode=paint_mode,
                          r_split=r_split, checkpoint_every=checkpoint_every,
                          coefficients=(kick, drift), engine=engine)


def density_mse(pos, target, paint_mode="atomic"):
    """Mean squared difference between the CIC density of ``pos`` and
    ``target`` (the loss of the reference's differentiable examples)."""
    rho = painting.cic_paint(torch.zeros_like(target), pos, mode=paint_mode)
    return ((rho - target)**2).mean()
