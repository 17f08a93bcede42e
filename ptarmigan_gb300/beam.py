"""Primary-beam generation, the host-side counterpart of ptarmigan's
``BeamBuilder::build`` (src/particle/builder.rs:173-219) and the Gaussian
parts of ``GammaDistribution``/``RadialDistribution``
(src/particle/dstr.rs:27-170).

The distributions are the reference's; the random numbers are numpy's
(seeded), so beams are statistically, not bitwise, equal to the reference's.
"""

import math

import numpy as np

from . import abi

C_LIGHT = 2.997925e8
ELECTRON_MASS_MEV = 0.510999


def initial_z(laser, sigma_z):
    """z0 = Field::ideal_initial_z() + 3 sigma_z (main.rs:1064)."""
    wavelength = laser.wavelength
    nc = laser.n_cycles
    if laser.envelope == abi.COS2:
        z = 0.5 * wavelength * nc
    elif laser.envelope == abi.FLATTOP:
        z = 0.5 * wavelength * (nc + 1.0)
    else:
        z = 2.0 * wavelength * nc
    return z + 3.0 * sigma_z


def build(n, gamma, sigma=0.0, radius=0.0, length=0.0, rms_div=0.0, laser=None, z0=None, species=abi.ELECTRON,
          energy_chirp=0.0, collision_angle=0.0, collision_plane=0.0, offset=(0.0, 0.0, 0.0),
          trunc_radius=None, uniform=False, stokes=(0.0, 0.0, 0.0), weight=1.0, seed=0, first_id=0):
    """Returns a dict of primary-particle arrays (abi.PARTICLE_FIELDS names).

    Arguments follow the YAML beam section: gamma/sigma (Lorentz factor mean
    and rms), radius (rms, or maximum when uniform), length (rms sigma_z),
    rms_divergence, energy_chirp, collision_angle/plane, offset.
    """
    rng = np.random.default_rng(seed)
    if z0 is None:
        z0 = initial_z(laser, length)
    rho = -energy_chirp  # builder.rs:120-124 flips the sign
    # GammaDistribution::Normal::sample, redrawn until gamma > 1 (dstr.rs:161-173)
    g = np.empty(n)
    dz = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        n0 = rng.standard_normal(todo.size)
        n1 = rng.standard_normal(todo.size)
        n2 = rho * n0 + math.sqrt(1.0 - rho * rho) * n1
        gg = gamma + sigma * n2
        ok = gg > 1.0
        g[todo[ok]] = gg[ok]
        dz[todo[ok]] = length * n0[ok]
        todo = todo[~ok]
    if species == abi.PHOTON:
        umag = -g
    else:
        umag = -np.sqrt(g * g - 1.0)
    theta_x = collision_angle + rms_div * rng.standard_normal(n)
    theta_y = rms_div * rng.standard_normal(n)
    ux = umag * np.sin(theta_x) * np.cos(theta_y)
    uy = umag * np.sin(theta_y)
    uz = umag * np.cos(theta_x) * np.cos(theta_y)
    c, s = math.cos(collision_plane), math.sin(collision_plane)
    ux, uy = c * ux - s * uy, c * uy + s * ux
    if species == abi.PHOTON:
        u0 = np.sqrt(ux * ux + uy * uy + uz * uz)
    else:
        u0 = np.sqrt(1.0 + ux * ux + uy * uy + uz * uz)
    if offset[2] >= 0.0:
        t = np.full(n, -z0)
        z = z0 + offset[2] + dz
    else:
        t = np.full(n, -z0 - abs(offset[2]))
        z = z0 + dz
    # RadialDistribution::sample (dstr.rs:27-51)
    if uniform:
        rr = radius * np.sqrt(rng.random(n))
        th = 2.0 * math.pi * rng.random(n)
        x, y = rr * np.cos(th), rr * np.sin(th)
    elif trunc_radius is not None:
        x = np.empty(n)
        y = np.empty(n)
        todo = np.arange(n)
        while todo.size:
            xx = radius * rng.standard_normal(todo.size)
            yy = radius * rng.standard_normal(todo.size)
            ok = xx * xx / trunc_radius ** 2 + yy * yy / trunc_radius ** 2 <= 1.0
            x[todo[ok]] = xx[ok]
            y[todo[ok]] = yy[ok]
            todo = todo[~ok]
    else:
        x = radius * rng.standard_normal(n)
        y = radius * rng.standard_normal(n)
    x = x + offset[0]
    y = y + offset[1]
    # r.rotate_around_y(angle) then rotate_around_z(plane)
    ca, sa = math.cos(collision_angle), math.sin(collision_angle)
    x, z = ca * x + sa * z, ca * z - sa * x
    x, y = c * x - s * y, c * y + s * x
    arrays = {
        "species": np.full(n, species, dtype=np.int32),
        "r": np.ascontiguousarray(np.stack([t, x, y, z], axis=1)),
        "u": np.ascontiguousarray(np.stack([u0, ux, uy, uz], axis=1)),
        "pol": np.ascontiguousarray(np.tile(np.array([1.0, *stokes]), (n, 1))),
        "weight": np.full(n, weight),
        "id": np.arange(first_id, first_id + n, dtype=np.uint64),
        "parent_id": np.arange(first_id, first_id + n, dtype=np.uint64),
    }
    return arrays


def gamma_from_energy(energy_gev):
    """Lorentz factor of an electron of the given total energy."""
    return energy_gev * 1.0e3 / ELECTRON_MASS_MEV
